// Prints the draws of the host Saru adapter (include/idpd/reference_api.hpp)
// for the seed triples read from stdin: per line "s1 s2 s3", the output line
// holds 4 u32() draws of one generator and nrml() of a fresh one.
#include <cstdio>

#include "idpd/reference_api.hpp"

int main() {
  unsigned a, b, c;
  while (std::scanf("%u %u %u", &a, &b, &c) == 3) {
    idpd::Saru g(a, b, c);
    unsigned u[4];
    for (int k = 0; k < 4; k++) u[k] = g.u32();
    idpd::Saru h(a, b, c);
    std::printf("%u %u %u %u %.17g\n", u[0], u[1], u[2], u[3], h.nrml());
  }
  return 0;
}
