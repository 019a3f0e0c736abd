// Runs the reference's main-loop body (src/main.cpp:166-184) through the C++
// adapters of include/idpd/reference_api.hpp on an FDPS-style particle system,
// then one ChemManager::RandomChemEvent, and writes the results for the
// Python side to compare with the oracle.
//
//   reference_api_run <in.bin> <out.bin> <nsteps>
//
// in.bin:  idpd_params (raw struct), uint32 n, n_amp, n_core, core_amp_id[n_core],
//          idpd_chem_params (raw struct), uint32 mt_seed, n_core_ptcl, core_ptcl_id[],
//          then n rows of pos[3], vel[3], acc[3] (double) and id, prop, amp_id, unit (uint32).
// out.bin: uint32 n_after_steps, rows (pos, vel, acc, density[3], press[3], delta_sumr[3],
//          nei_cm[6]), bonded virial of every step (3 doubles each), then the event:
//          int32 cont, uint32 amp_num, uint32 n_after_event, the new rows (pos, vel,
//          id, prop, amp_id, unit), uint32 len(glob_topol), glob_topol.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "particle_simulator.hpp"
#include "idpd/reference_api.hpp"

namespace {

// The FPDPD fields the adapters read and write (ptcl_class.hpp:29-35).
struct FP {
  PS::F64vec pos, vel, acc, press, delta_sumr;
  PS::F64vec nei_cm_pos[2];
  double density[3] = {0.0, 0.0, 0.0};
  uint32_t id = 0, prop = 0, amp_id = 0, unit = 0;
};

// Parameter members ChemManager reads (parameter.hpp:230-243).
struct ChemParam {
  double p_thresld, eps, influ_rad, influ_hei, influ_dep, influ_grd;
  uint32_t amp_num, max_amp_num;
  std::vector<uint32_t> core_ptcl_id;
};

template <class T>
void rd(FILE* f, T* p, size_t n = 1) {
  if (std::fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short input\n");
    std::exit(2);
  }
}
template <class T>
void wr(FILE* f, const T* p, size_t n = 1) {
  std::fwrite(p, sizeof(T), n, f);
}
void wr3(FILE* f, const PS::F64vec& v) {
  const double a[3] = {v.x, v.y, v.z};
  wr(f, a, 3);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s in.bin out.bin nsteps\n", argv[0]);
    return 2;
  }
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  idpd_params p;
  rd(in, &p);
  uint32_t n, n_amp, n_core;
  rd(in, &n);
  rd(in, &n_amp);
  rd(in, &n_core);
  std::vector<uint32_t> core(n_core);
  if (n_core) rd(in, core.data(), n_core);
  idpd_chem_params cp;
  rd(in, &cp);
  uint32_t mt_seed, n_core_ptcl;
  rd(in, &mt_seed);
  rd(in, &n_core_ptcl);
  std::vector<uint32_t> core_ptcl(n_core_ptcl);
  if (n_core_ptcl) rd(in, core_ptcl.data(), n_core_ptcl);
  PS::ParticleSystem<FP> sys;
  sys.setNumberOfParticleLocal((PS::S32)n);
  for (uint32_t i = 0; i < n; i++) {
    double a[9];
    uint32_t u[4];
    rd(in, a, 9);
    rd(in, u, 4);
    sys[i].pos = PS::F64vec(a[0], a[1], a[2]);
    sys[i].vel = PS::F64vec(a[3], a[4], a[5]);
    sys[i].acc = PS::F64vec(a[6], a[7], a[8]);
    sys[i].id = u[0];
    sys[i].prop = u[1];
    sys[i].amp_id = u[2];
    sys[i].unit = u[3];
  }
  std::fclose(in);
  const int nsteps = std::atoi(argv[3]);

  uint32_t time = p.time;  // Parameter::time
  idpd::Session session(p, &time);
  idpd::bind(sys, session);
  idpd::ForceBonded<PS::ParticleSystem<FP>> fbonded(sys, 4 * (n_amp + 1024), n_amp, core);
  const PS::F64vec box(p.box[0], p.box[1], p.box[2]);
  const PS::F64vec ibox(1.0 / p.box[0], 1.0 / p.box[1], 1.0 / p.box[2]);
  std::vector<PS::F64vec> virs;
  for (int s = 0; s < nsteps; s++, time++) {
    idpd::drift_and_predict(sys, p.dt, box, ibox);
    idpd::calcForceAllAndWriteBack(idpd::CalcDensity(), sys);
    idpd::calcForceAllAndWriteBack(idpd::CalcForceEpEpDPD(), sys);
    PS::F64vec vir;
    fbonded.CalcListedForce(sys, vir);
    virs.push_back(vir);
    idpd::kick(sys, p.dt);
    if (time % 100 == 0) idpd::remove_cmdrift_global(sys);
  }

  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  const uint32_t n1 = (uint32_t)sys.getNumberOfParticleLocal();
  wr(out, &n1);
  for (uint32_t i = 0; i < n1; i++) {
    wr3(out, sys[i].pos);
    wr3(out, sys[i].vel);
    wr3(out, sys[i].acc);
    wr(out, sys[i].density, 3);
    wr3(out, sys[i].press);
    wr3(out, sys[i].delta_sumr);
    wr3(out, sys[i].nei_cm_pos[0]);
    wr3(out, sys[i].nei_cm_pos[1]);
  }
  for (const auto& v : virs) wr3(out, v);

  ChemParam param{cp.p_thresld, cp.eps, cp.influ_rad, cp.influ_hei, cp.influ_dep, cp.influ_grd,
                  cp.amp_num, cp.max_amp_num, core_ptcl};
  idpd::ChemManager<FP> chem(mt_seed, 1024);
  std::vector<uint32_t> glob_topol = fbonded.glob_topol();
  const int32_t cont = chem.RandomChemEvent(sys, glob_topol, param) ? 1 : 0;
  const uint32_t n2 = (uint32_t)sys.getNumberOfParticleLocal();
  wr(out, &cont);
  wr(out, &param.amp_num);
  wr(out, &n2);
  for (uint32_t i = n1; i < n2; i++) {
    wr3(out, sys[i].pos);
    wr3(out, sys[i].vel);
    const uint32_t u[4] = {sys[i].id, sys[i].prop, sys[i].amp_id, sys[i].unit};
    wr(out, u, 4);
  }
  const uint32_t nt = (uint32_t)glob_topol.size();
  wr(out, &nt);
  wr(out, glob_topol.data(), nt);
  std::fclose(out);
  idpd::unbind(sys);
  return 0;
}
