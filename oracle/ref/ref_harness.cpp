// Harness that compiles the reference's own hot-path headers, unmodified, into
// a shared library with a C ABI, so that the C restatement in oracle/ can be
// pinned against the reference itself and golden vectors can be written.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the
// headers under the reference checkout; never part of the product.
//
// The FDPS tree gather (src/main.cpp:173-174) is replaced by a cell-list
// gatherer: each i-group is one cell of a grid with cells >= search_rad (1.2),
// and its j list is every particle of the 27 surrounding cells with its
// periodic image position (a superset of the search sphere, self included),
// cells visited dz-major, dy, dx from -1 to 1, particles in ascending index.
// The C restatement gathers in the same order, so FP64 sums agree bit for bit.

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "particle_simulator.hpp"
#include "user_defs.h"
#include "parameter.hpp"
#include "f_calculator.hpp"
#include "driftkick.hpp"
#ifdef CHEM_MODE
#include "chemmanager.hpp"
#endif

// Static members that the reference's driver defines (src/main.cpp:27-31).
constexpr char Parameter::atom_type[21];
PS::F64vec Parameter::box_leng, Parameter::ibox_leng;
PS::U32 Parameter::time;
PS::U32 Parameter::all_time, Parameter::step_mic, Parameter::step_mac;

namespace {

PS::ParticleSystem<FPDPD> g_sys;
Parameter* g_param = nullptr;
ForceBonded<PS::ParticleSystem<FPDPD> >* g_bonded = nullptr;

Parameter& param() {
  if (!g_param) {
    g_param = new Parameter(".");
    g_param->Initialize();
  }
  return *g_param;
}

struct CellGrid {
  int nc[3];
  std::vector<int> start, members;
};

// Cells of at least search_rad on a side; particles in ascending index.
void build_cells(CellGrid& g) {
  const int n = g_sys.getNumberOfParticleLocal();
  double inv[3];
  for (int d = 0; d < 3; d++) {
    g.nc[d] = (int)(Parameter::box_leng[d] / Parameter::search_rad);
    inv[d] = g.nc[d] / Parameter::box_leng[d];
  }
  const int ncell = g.nc[0] * g.nc[1] * g.nc[2];
  std::vector<int> cid(n), cnt(ncell + 1, 0);
  for (int i = 0; i < n; i++) {
    int c[3];
    for (int d = 0; d < 3; d++) {
      c[d] = (int)(g_sys[i].pos[d] * inv[d]);
      if (c[d] < 0) c[d] = 0;
      if (c[d] >= g.nc[d]) c[d] = g.nc[d] - 1;
    }
    cid[i] = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
    cnt[cid[i] + 1]++;
  }
  for (int c = 0; c < ncell; c++) cnt[c + 1] += cnt[c];
  g.start = cnt;
  g.members.assign(n, 0);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; i++) g.members[fill[cid[i]]++] = i;
}

template <class EPI, class EPJ, class RES, class F>
void gather_and_call(F func) {
  CellGrid g;
  build_cells(g);
  const int ncell = g.nc[0] * g.nc[1] * g.nc[2];
  std::vector<EPI> epi;
  std::vector<EPJ> epj;
  std::vector<RES> res;
  for (int cz = 0; cz < g.nc[2]; cz++)
    for (int cy = 0; cy < g.nc[1]; cy++)
      for (int cx = 0; cx < g.nc[0]; cx++) {
        const int c = (cz * g.nc[1] + cy) * g.nc[0] + cx;
        const int ni = g.start[c + 1] - g.start[c];
        if (ni == 0) continue;
        epi.resize(ni);
        res.resize(ni);
        for (int k = 0; k < ni; k++) {
          epi[k].copyFromFP(g_sys[g.members[g.start[c] + k]]);
          res[k].clear();
        }
        epj.clear();
        for (int dz = -1; dz <= 1; dz++)
          for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
              const int q[3] = {cx + dx, cy + dy, cz + dz};
              int w[3];
              double sh[3];
              for (int d = 0; d < 3; d++) {
                int s = q[d] < 0 ? -1 : (q[d] >= g.nc[d] ? 1 : 0);
                w[d] = q[d] - s * g.nc[d];
                sh[d] = (double)s * Parameter::box_leng[d];
              }
              const int cj = (w[2] * g.nc[1] + w[1]) * g.nc[0] + w[0];
              for (int m = g.start[cj]; m < g.start[cj + 1]; m++) {
                EPJ e;
                e.copyFromFP(g_sys[g.members[m]]);
                PS::F64vec p = g_sys[g.members[m]].pos;
                p.x = p.x + sh[0];
                p.y = p.y + sh[1];
                p.z = p.z + sh[2];
                e.setPos(p);
                epj.push_back(e);
              }
            }
        func(epi.data(), ni, epj.data(), (int)epj.size(), res.data());
        for (int k = 0; k < ni; k++) g_sys[g.members[g.start[c] + k]].copyFromForce(res[k]);
      }
  (void)ncell;
}

}  // namespace

extern "C" {

int ref_is_pairwise() {
#ifdef PAIRWISE_DPD
  return 1;
#else
  return 0;
#endif
}

// Parses <dir>/run_param.txt with Parameter::LoadParam (parameter.hpp:378-387),
// which also derives the MDPD tables (CalcInterCoef, parameter.hpp:138-186).
void ref_load_params(const char* dir) {
  delete g_param;
  g_param = new Parameter(std::string(dir));
  g_param->Initialize();
  g_param->LoadParam();
}

void ref_get_tables(double* cf_c, double* cf_g, double* cf_r, double* cf_m, double* scal) {
  std::memcpy(cf_c, &Parameter::cf_c[0][0], 9 * sizeof(double));
  std::memcpy(cf_g, &Parameter::cf_g[0][0], 9 * sizeof(double));
  std::memcpy(cf_r, &Parameter::cf_r[0][0], 9 * sizeof(double));
  std::memcpy(cf_m, &Parameter::cf_m[0][0][0], 27 * sizeof(double));
  scal[0] = Parameter::cf_s;
  scal[1] = Parameter::cf_b;
  scal[2] = Parameter::cf_b_rigid;
  scal[3] = Parameter::box_leng.x;
  scal[4] = Parameter::box_leng.y;
  scal[5] = Parameter::box_leng.z;
  scal[6] = param().dt;
  scal[7] = param().chi;
  scal[8] = param().kappa;
  scal[9] = param().rho_co;
}

void ref_set_tables(const double* cf_c, const double* cf_g, const double* cf_r, const double* cf_m,
                    double cf_s, double cf_b, double cf_b_rigid, const double* box) {
  param();
  std::memcpy(&Parameter::cf_c[0][0], cf_c, 9 * sizeof(double));
  std::memcpy(&Parameter::cf_g[0][0], cf_g, 9 * sizeof(double));
  std::memcpy(&Parameter::cf_r[0][0], cf_r, 9 * sizeof(double));
  std::memcpy(&Parameter::cf_m[0][0][0], cf_m, 27 * sizeof(double));
  Parameter::cf_s = cf_s;
  Parameter::cf_b = cf_b;
  Parameter::cf_b_rigid = cf_b_rigid;
  for (int d = 0; d < 3; d++) {
    Parameter::box_leng[d] = box[d];
    Parameter::ibox_leng[d] = 1.0 / box[d];
  }
}

void ref_set_seed_time(uint32_t seed, uint32_t time) {
  CalcForceEpEpDPD::m_seed = seed;
  Parameter::time = time;
}

void ref_saru_u32(uint32_t s1, uint32_t s2, uint32_t s3, int count, uint32_t* out) {
  Saru s(s1, s2, s3);
  for (int k = 0; k < count; k++) out[k] = s.u32();
}

double ref_saru_nrml(uint32_t s1, uint32_t s2, uint32_t s3) {
  Saru s(s1, s2, s3);
  return s.nrml();
}

double ref_saru_uni_open(uint32_t s1, uint32_t s2, uint32_t s3, int draw) {
  Saru s(s1, s2, s3);
  double v = 0.0;
  for (int k = 0; k <= draw; k++) v = s.uni_open();
  return v;
}

// Particle state in FPDPD rows (ptcl_class.hpp:29-35).
void ref_sys_set(int n, const double* pos, const double* vel, const double* acc, const uint32_t* id,
                 const uint32_t* prop, const uint32_t* amp_id, const uint32_t* unit) {
  g_sys.setNumberOfParticleLocal(n);
  for (int i = 0; i < n; i++) {
    FPDPD& p = g_sys[i];
    p.id = id[i];
    p.prop = prop[i];
    p.amp_id = amp_id[i];
    p.unit = unit[i];
    for (int d = 0; d < 3; d++) {
      p.pos[d] = pos[3 * i + d];
      p.vel[d] = vel[3 * i + d];
      p.acc[d] = acc[3 * i + d];
      p.vel_buf[d] = vel[3 * i + d];
    }
    p.delta_sumr = 0.0;
    p.press = 0.0;
    p.nei_cm_pos[0] = p.nei_cm_pos[1] = 0.0;
    p.density.fill(0.0);
  }
}

int ref_sys_n() { return g_sys.getNumberOfParticleLocal(); }

void ref_sys_get(double* pos, double* vel, double* vel_buf, double* acc, double* press, double* dens,
                 double* nei_cm, double* dsr, uint32_t* id, uint32_t* prop, uint32_t* amp_id,
                 uint32_t* unit) {
  const int n = g_sys.getNumberOfParticleLocal();
  for (int i = 0; i < n; i++) {
    const FPDPD& p = g_sys[i];
    for (int d = 0; d < 3; d++) {
      pos[3 * i + d] = p.pos[d];
      vel[3 * i + d] = p.vel[d];
      vel_buf[3 * i + d] = p.vel_buf[d];
      acc[3 * i + d] = p.acc[d];
      press[3 * i + d] = p.press[d];
      dens[3 * i + d] = p.density[d];
      nei_cm[6 * i + d] = p.nei_cm_pos[0][d];
      nei_cm[6 * i + 3 + d] = p.nei_cm_pos[1][d];
      dsr[3 * i + d] = p.delta_sumr[d];
    }
    id[i] = p.id;
    prop[i] = p.prop;
    amp_id[i] = p.amp_id;
    unit[i] = p.unit;
  }
}

void ref_sys_set_density(const double* dens) {
  const int n = g_sys.getNumberOfParticleLocal();
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) g_sys[i].density[k] = dens[3 * i + k];
}

void ref_sys_set_vel_buf(const double* vb) {
  const int n = g_sys.getNumberOfParticleLocal();
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) g_sys[i].vel_buf[d] = vb[3 * i + d];
}

// Pass 1 (nbdf_calculator.hpp:11-60) + write-back (ptcl_class.hpp:53-57).
void ref_density() {
  gather_and_call<EPI::Density, EPJ::Density, RESULT::Density>(CalcDensity());
}

// Pass 2 (nbdf_calculator.hpp:63-145) + write-back (ptcl_class.hpp:48-51).
void ref_force() {
  gather_and_call<EPI::DPD, EPJ::DPD, RESULT::ForceDPD>(CalcForceEpEpDPD());
}

// ForceBonded construction (bdf_calculator.hpp:32-51) over the current state.
void ref_bonded_init(uint32_t init_amp_num, int n_core, const uint32_t* core_amp_id) {
  delete g_bonded;
  std::vector<PS::U32> core(core_amp_id, core_amp_id + n_core);
  g_bonded = new ForceBonded<PS::ParticleSystem<FPDPD> >(g_sys, Parameter::all_unit * init_amp_num,
                                                         init_amp_num, core);
}

// ForceBonded::CalcListedForce (bdf_calculator.hpp:191-220): acc += bonded.
void ref_bonded(double* vir) {
  PS::F64vec v(0.0, 0.0, 0.0);
  g_bonded->CalcListedForce(g_sys, v);
  vir[0] = v.x;
  vir[1] = v.y;
  vir[2] = v.z;
}

int ref_topol(uint32_t* out, int cap) {
  PS::ReallocatableArray<PS::U32>& t = g_bonded->glob_topol();
  for (int i = 0; i < t.size() && i < cap; i++) out[i] = t[i];
  return t.size();
}

void ref_drift(double dt) {
  drift_and_predict(g_sys, dt, Parameter::box_leng, Parameter::ibox_leng);
}

void ref_kick(double dt) { kick(g_sys, dt); }

void ref_cmdrift() { remove_cmdrift_global(g_sys); }

// One iteration of the main loop body (src/main.cpp:166-184) without the
// domain-decomposition, chemistry and observer calls.
void ref_md_step(double dt, double* bonded_vir) {
  drift_and_predict(g_sys, dt, Parameter::box_leng, Parameter::ibox_leng);
  ref_density();
  ref_force();
  PS::F64vec v(0.0, 0.0, 0.0);
  if (g_bonded) g_bonded->CalcListedForce(g_sys, v);
  bonded_vir[0] = v.x;
  bonded_vir[1] = v.y;
  bonded_vir[2] = v.z;
  kick(g_sys, dt);
  if (Parameter::time % Parameter::cm_corr == 0) remove_cmdrift_global(g_sys);
  Parameter::time++;
}

#ifdef CHEM_MODE
// One ChemManager::RandomChemEvent (single-node, chemmanager.hpp:244-281)
// with LOCAL_CHEM_EVENT, from a fresh ChemManager seeded with `mt_seed`.
// Returns 1 to continue, 0 to stop; new particles are appended to the state.
int ref_chem_event(uint32_t mt_seed, double p_thresld, double eps, uint32_t amp_num,
                   uint32_t max_amp_num, double influ_rad, double influ_hei, double influ_dep,
                   double influ_grd, int n_core, const uint32_t* core_amp_id,
                   const uint32_t* core_ptcl_id, uint32_t* amp_num_out) {
  Parameter& p = param();
  p.p_thresld = p_thresld;
  p.eps = eps;
  p.amp_num = amp_num;
  p.max_amp_num = max_amp_num;
  p.influ_rad = influ_rad;
  p.influ_hei = influ_hei;
  p.influ_dep = influ_dep;
  p.influ_grd = influ_grd;
  p.core_amp_id_.assign(core_amp_id, core_amp_id + n_core);
  p.core_ptcl_id.assign(core_ptcl_id, core_ptcl_id + n_core);
  ChemManager<FPDPD> cm(mt_seed);
  const bool cont = cm.RandomChemEvent(g_sys, g_bonded->glob_topol(), p);
  *amp_num_out = p.amp_num;
  return cont ? 1 : 0;
}

// MT19937 draws of the stand-in PS::MT, for pinning the C restatement.
void ref_mt_draws(uint32_t seed, int n, uint32_t* out) {
  PS::MT::init_genrand(seed);
  for (int i = 0; i < n; i++) out[i] = PS::MT::genrand_int32();
}
#endif

}  // extern "C"
