// The reference's on-disk formats on the host: run_param.txt (tag / value
// lines, parameter.hpp:352-387) and the xyz particle files (io_util.hpp:26-31,
// 95-129; ptcl_class.hpp:60-86).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "idpd_engine.h"

namespace idpd {
void set_library_error(const char* msg);
}

namespace {

constexpr double kPi = 3.14159265358979323846;
// Parameter::atom_type (parameter.hpp:207-209): the letter written per property.
constexpr char kAtomType[21] = {'O', 'N', 'C', 'S', 'P', 'Z', 'X', 'O', 'N', 'C', 'S',
                                'P', 'Z', 'X', 'O', 'N', 'C', 'S', 'P', 'Z', 'X'};

int fmt_fail(int code, const std::string& msg) {
  idpd::set_library_error(msg.c_str());
  return code;
}

using TagMap = std::map<std::string, std::vector<std::string>>;

// ReadTagValues (parameter.hpp:352-376): ';' comments, blank lines skipped,
// leading / trailing blanks removed, the first word is the tag.
TagMap read_tags(std::ifstream& in) {
  TagMap m;
  std::string line;
  while (std::getline(in, line)) {
    const size_t c = line.find(';');
    if (c != std::string::npos) line = line.substr(0, c);
    std::stringstream ss(line);
    std::string tag;
    if (!(ss >> tag)) continue;
    std::vector<std::string> vals;
    std::string v;
    while (ss >> v) vals.push_back(v);
    m[tag] = vals;
  }
  return m;
}

bool have(const TagMap& m, const char* tag, size_t n) {
  auto it = m.find(tag);
  return it != m.end() && it->second.size() == n;
}

// std::stof semantics: the decimal text rounded to float, then widened.
bool real(const TagMap& m, const char* tag, size_t n, double* out) {
  if (!have(m, tag, n)) return false;
  for (size_t k = 0; k < n; k++) out[k] = (double)std::stof(m.at(tag)[k]);
  return true;
}

bool uinteger(const TagMap& m, const char* tag, size_t n, uint32_t* out) {
  if (!have(m, tag, n)) return false;
  for (size_t k = 0; k < n; k++) out[k] = (uint32_t)std::stoi(m.at(tag)[k]);
  return true;
}

}  // namespace

extern "C" {

int idpd_read_run_param(const char* path, idpd_run_file* out) {
  if (!path || !out) return fmt_fail(IDPD_ERR_INVALID_ARG, "null pointer");
  std::ifstream in(path);
  if (!in) return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": cannot open");
  TagMap m;
  try {
    m = read_tags(in);
  } catch (...) {
    return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": read error");
  }
  std::memset(out, 0, sizeof(*out));
  const double nan = std::nan("");
  idpd_run_param& rp = out->rp;
  rp.vbb = 0.1;  // Parameter::vbb default (parameter.hpp:226)
  try {
    struct Req { const char* tag; size_t n; double* d; uint32_t* u; };
    const Req req[] = {
        {"box_leng", 3, rp.box, nullptr},    {"init_amp_num", 1, nullptr, &out->init_amp_num},
        {"sol_num", 1, nullptr, &out->sol_num}, {"dt", 1, &rp.dt, nullptr},
        {"cf_r", 6, rp.cf_r_upper, nullptr}, {"cf_s", 1, &rp.cf_s, nullptr},
        {"cf_b", 1, &rp.cf_b, nullptr},      {"cf_b_rigid", 1, &rp.cf_b_rigid, nullptr},
        {"chi", 1, &rp.chi, nullptr},        {"kappa", 1, &rp.kappa, nullptr},
        {"rho_co", 1, &rp.rho_co, nullptr},  {"all_time", 1, nullptr, &out->all_time},
        {"step_mic", 1, nullptr, &out->step_mic}, {"step_mac", 1, nullptr, &out->step_mac},
    };
    for (const Req& r : req) {
      const bool ok = r.d ? real(m, r.tag, r.n, r.d) : uinteger(m, r.tag, r.n, r.u);
      if (!ok)
        return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": tag " + r.tag +
                                                  " missing or with the wrong number of values");
    }
    if (m.count("vbb")) real(m, "vbb", 1, &rp.vbb);
    // reaction block (MatchingTagValues :102-135)
    idpd_chem_params& c = out->chem;
    c.amp_num = out->init_amp_num;
    out->influ_vol = out->upside_rad = nan;
    bool chem = real(m, "p_thresld", 1, &c.p_thresld) && real(m, "eps", 1, &c.eps) &&
                uinteger(m, "max_amp_num", 1, &c.max_amp_num) &&
                real(m, "influ_hei", 1, &c.influ_hei) && real(m, "influ_dep", 1, &c.influ_dep);
    if (chem && m.count("influ_vol")) {
      chem = real(m, "influ_vol", 1, &out->influ_vol) && real(m, "upside_rad", 1, &out->upside_rad);
      if (chem) {  // CalcInfluGrdAndRad (:42-56)
        const double hei_sum = c.influ_hei + c.influ_dep;
        const double up = out->upside_rad;
        const double val = 12.0 * out->influ_vol / (kPi * hei_sum) - 3.0 * up * up;
        if (val > 0.0) {
          const double down = (std::sqrt(val) - up) * 0.5;
          c.influ_grd = (down - up) / hei_sum;
        } else {
          const double hei_new = 3.0 * out->influ_vol / (kPi * up * up);
          c.influ_grd = -up / hei_new;
        }
        c.influ_rad = up + c.influ_grd * c.influ_hei;
      }
    } else if (chem) {
      chem = real(m, "influ_rad", 1, &c.influ_rad) && real(m, "influ_grd", 1, &c.influ_grd);
      if (chem) {  // CalcInfluVol (:58-72)
        const double hei_sum = c.influ_hei + c.influ_dep;
        const double up = c.influ_rad - c.influ_grd * c.influ_hei;
        const double down = c.influ_rad + c.influ_grd * c.influ_dep;
        if (down >= 0.0) {
          const double ua = kPi * up * up, da = kPi * down * down;
          out->influ_vol = (ua + da + std::sqrt(da * ua)) * hei_sum / 3.0;
        } else {
          const double hei_new = -up / c.influ_grd;
          out->influ_vol = kPi * up * up * hei_new / 3.0;
        }
      }
    }
    auto it = m.find("core_amp_id");
    if (chem && it != m.end() && !it->second.empty()) {
      out->n_core = (int32_t)it->second.size();
      for (int32_t k = 0; k < out->n_core && k < IDPD_CHEM_MAX_CORE; k++)
        out->core_amp_id[k] = (uint32_t)std::stoi(it->second[k]);
    } else {
      chem = false;
    }
    out->has_chem = chem ? 1 : 0;
  } catch (...) {
    return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": a value is not a number");
  }
  return IDPD_OK;
}

int idpd_read_xyz(const char* path, int32_t cap, int32_t* n, uint32_t* time, double* pos,
                  double* vel, double* vel_buf, double* acc, uint32_t* id, uint32_t* prop,
                  uint32_t* amp_id, uint32_t* unit) {
  if (!path || !n || cap < 0) return fmt_fail(IDPD_ERR_INVALID_ARG, "bad argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": cannot open");
  unsigned num = 0, t = 0;
  char word[16] = {0};
  if (std::fscanf(f, "%u\n", &num) != 1 || std::fscanf(f, "%15s %u\n", word, &t) != 2 ||
      std::strcmp(word, "time") != 0) {
    std::fclose(f);
    return fmt_fail(IDPD_ERR_INVALID_ARG,
                    std::string(path) + ": header must be '<number of particles>' and 'time <t>'");
  }
  if ((long long)num > cap) {
    std::fclose(f);
    return fmt_fail(IDPD_ERR_CAPACITY, std::string(path) + ": more particles than the buffers hold");
  }
  for (unsigned i = 0; i < num; i++) {
    char type;
    double r[3], v[3], vb[3], a[3];
    unsigned u[4];
    const int got = std::fscanf(f, " %c %lf %lf %lf %u %u %u %u %lf %lf %lf %lf %lf %lf %lf %lf %lf",
                                &type, &r[0], &r[1], &r[2], &u[0], &u[1], &u[2], &u[3], &v[0],
                                &v[1], &v[2], &vb[0], &vb[1], &vb[2], &a[0], &a[1], &a[2]);
    if (got != 17) {
      std::fclose(f);
      return fmt_fail(IDPD_ERR_INVALID_ARG,
                      std::string(path) + ": row " + std::to_string(i) + " is malformed or missing");
    }
    for (int k = 0; k < 3; k++) {
      if (pos) pos[3 * (size_t)i + k] = r[k];
      if (vel) vel[3 * (size_t)i + k] = v[k];
      if (vel_buf) vel_buf[3 * (size_t)i + k] = vb[k];
      if (acc) acc[3 * (size_t)i + k] = a[k];
    }
    if (id) id[i] = u[0];
    if (prop) prop[i] = u[1];
    if (amp_id) amp_id[i] = u[2];
    if (unit) unit[i] = u[3];
  }
  char extra;
  const bool more = std::fscanf(f, " %c", &extra) == 1;
  std::fclose(f);
  if (more)
    return fmt_fail(IDPD_ERR_INVALID_ARG,
                    std::string(path) + ": more rows than the header's particle count");
  *n = (int32_t)num;
  if (time) *time = t;
  return IDPD_OK;
}

int idpd_write_xyz(const char* path, int32_t append, uint32_t time, int32_t n, const double* pos,
                   const double* vel, const double* vel_buf, const double* acc,
                   const uint32_t* id, const uint32_t* prop, const uint32_t* amp_id,
                   const uint32_t* unit) {
  if (!path || n < 0 || (n > 0 && (!pos || !vel || !acc || !id || !prop || !amp_id || !unit)))
    return fmt_fail(IDPD_ERR_INVALID_ARG, "bad argument");
  FILE* f = std::fopen(path, append ? "a" : "w");
  if (!f) return fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": cannot open");
  std::fprintf(f, "%u\n", (unsigned)n);
  std::fprintf(f, "time %u\n", time);
  for (int32_t i = 0; i < n; i++) {
    const double* r = pos + 3 * (size_t)i;
    const double* v = vel + 3 * (size_t)i;
    const double* vb = vel_buf ? vel_buf + 3 * (size_t)i : v;
    const double* a = acc + 3 * (size_t)i;
    const char type = prop[i] < 21u ? kAtomType[prop[i]] : 'X';
    std::fprintf(f,
                 "%c %.15g %.15g %.15g %u %u %u %u %.15g %.15g %.15g %.15g %.15g %.15g %.15g "
                 "%.15g %.15g\n",
                 type, r[0], r[1], r[2], id[i], prop[i], amp_id[i], unit[i], v[0], v[1], v[2],
                 vb[0], vb[1], vb[2], a[0], a[1], a[2]);
  }
  const bool ok = std::fclose(f) == 0;
  return ok ? IDPD_OK : fmt_fail(IDPD_ERR_INVALID_ARG, std::string(path) + ": write error");
}

}  // extern "C"
