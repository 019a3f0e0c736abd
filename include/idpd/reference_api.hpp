// C++ adapters with the reference's driver-level names over the C ABI of
// idpd_engine.h, so that a host built around an FDPS-style particle system
// can call the GPU engine where it calls the reference's CPU code:
//
//   reference (include/...)                          adapter (namespace idpd)
//   drift_and_predict(sys, dt, box, ibox)            drift_and_predict(sys, dt, box, ibox)
//     driftkick.hpp:6-27
//   kick(sys, dt)                driftkick.hpp:33-40 kick(sys, dt)
//   remove_cmdrift_global(sys)   driftkick.hpp:43-54 remove_cmdrift_global(sys)
//   dens_tree.calcForceAllAndWriteBack(CalcDensity(), sys, dinfo)
//     main.cpp:173, nbdf_calculator.hpp:11-60       calcForceAllAndWriteBack(CalcDensity(), sys)
//   force_tree.calcForceAllAndWriteBack(CalcForceEpEpDPD(), sys, dinfo)
//     main.cpp:174, nbdf_calculator.hpp:63-147      calcForceAllAndWriteBack(CalcForceEpEpDPD(), sys)
//   ForceBonded<Tpsys>(sys, buf_size, amp_num, core_amp_id), CalcListedForce(sys, vir),
//   glob_topol(), ExpandTopolBuffer(n)  bdf_calculator.hpp:16-51,90-92,191-220
//                                                    ForceBonded<Tpsys> (same members)
//   ChemManager<FP>(seed), RandomChemEvent(sys, glob_topol, param), h2t_vecs(),
//   core_poss_h()  chemmanager.hpp:176-189,244-281  ChemManager<FP> (same members)
//   Saru(s1, s2, s3), u32(), uni_open(), nrml()
//     saruprng.hpp:89,114,123-125,239-255,322-333,427-445
//                                                    Saru (host, same members)
//
// The particle system is duck-typed like FDPS's ParticleSystem<FPDPD>:
// sys.getNumberOfParticleLocal(), sys[i].{pos, vel, acc, press, delta_sumr}
// (vectors with .x .y .z), sys[i].density[3], sys[i].nei_cm_pos[2],
// sys[i].{id, prop, amp_id, unit}, and sys.AddNewParticle(p) for the reaction.
// Parameter-like objects need the members ChemManager reads (p_thresld, eps,
// influ_rad, influ_hei, influ_dep, influ_grd, amp_num, max_amp_num,
// core_ptcl_id).
//
// A Session is one engine handle mirroring one particle system; bind() ties
// them so that the free functions keep the reference's signatures. Each
// adapter call pushes the host state the engine needs, runs the pass on the
// GPU and writes back what the reference's call writes, so the host state
// stays authoritative; a host that wants the full GPU speed calls
// idpd_step() on the session's handle instead.
//
// Errors end the program, as PS::Abort does in the reference, after printing
// the engine's message (no exception crosses the C ABI).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "idpd_engine.h"

namespace idpd {

inline void check(const idpd_handle* h, int rc, const char* what) {
  if (rc == IDPD_OK) return;
  char msg[512];
  idpd_last_error(h, msg, sizeof(msg));
  std::fprintf(stderr, "idpd: %s failed (status %d): %s\n", what, rc, msg);
  std::abort();
}

// Saru on the host (saruprng.hpp:83-445): the 3-seed constructor, u32(),
// uni_open() and nrml() with the reference's semantics, for host code that
// draws from the same counter-based streams as the pair kernels. The integer
// draws are bit-exact with the reference; uni_open() and nrml() are its FP64
// expressions (nrml draws its logarithm's argument first, as the reference's
// build evaluates sqrt(-2 log(uni_open())) * cos(2 pi uni_open())).
class Saru {
 public:
  Saru(uint32_t a, uint32_t b, uint32_t c) {
    // the seeding hash of saruprng.hpp:239-255
    c ^= (a << 7) ^ (b >> 6);
    b += (a >> 4) ^ (c >> 15);
    a ^= (b << 9) + (c << 8);
    c ^= 0xA5366B4Du * ((b >> 11) ^ (a << 1));
    b += 0x72BE1579u * ((a << 4) ^ (c >> 16));
    a ^= 0x3F38A6EDu * ((c >> 5) ^ sar(b, 22));
    b += a * c;
    a += c ^ (b >> 2);
    b ^= sar(b, 17);
    lcg_ = 0x79dedea3u * (a ^ sar(a, 14));
    weyl_ = (lcg_ + b) ^ sar(lcg_, 8);
    lcg_ = lcg_ + (weyl_ * (weyl_ ^ 0xdddf97f5u));
    weyl_ = 0xABCB96F7u + (weyl_ >> 1);
  }
  // one LCG and Weyl step, then the output mix (saruprng.hpp:173-177,199-202,322-333)
  uint32_t u32() {
    lcg_ = 0x4beb5d59u * lcg_ + 0x2600e1f7u;
    weyl_ = weyl_ + 0x8009d14bu + (sar(weyl_, 31) & 0xda879addu);
    const uint32_t v = (lcg_ ^ (lcg_ >> 26)) + weyl_;
    return (v ^ (v >> 20)) * 0x6957f5a7u;
  }
  // (0, 1) from 31 bits (saruprng.hpp:427-434)
  double uni_open() {
    return ((double)(int32_t)(u32() >> 1) + 0.5) * (1.0 / 2147483648.0);
  }
  // Box-Muller normal (saruprng.hpp:442-445)
  double nrml() {
    const double u1 = uni_open();
    const double u2 = uni_open();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
  }

 private:
  static uint32_t sar(uint32_t x, int s) { return (uint32_t)((int32_t)x >> s); }
  uint32_t lcg_, weyl_;
};

class Session {
 public:
  // p: the replica's parameters (idpd_derive_params + seed); time: the
  // host's step counter (Parameter::time), read before every pass that uses it.
  Session(const idpd_params& p, const uint32_t* time, int device = 0) : p_(p), time_(time) {
    idpd_config cfg = {};
    cfg.n_replicas = 1;
    cfg.device = device;
    check(nullptr, idpd_create(&cfg, &h_), "idpd_create");
    check(h_, idpd_set_params(h_, 0, &p_), "idpd_set_params");
  }
  ~Session() { idpd_destroy(h_); }
  Session(const Session&) = delete;
  Session& operator=(const Session&) = delete;

  idpd_handle* handle() { return h_; }

  // Full upload of the particle rows (ids, properties, molecules).
  template <class Tpsys>
  void upload(const Tpsys& sys) {
    const int n = (int)sys.getNumberOfParticleLocal();
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), acc(3 * (size_t)n);
    std::vector<uint32_t> id(n), prop(n), amp(n), unit(n);
    for (int i = 0; i < n; i++) {
      put3(&pos[3 * (size_t)i], sys[i].pos);
      put3(&vel[3 * (size_t)i], sys[i].vel);
      put3(&acc[3 * (size_t)i], sys[i].acc);
      id[i] = sys[i].id;
      prop[i] = sys[i].prop;
      amp[i] = sys[i].amp_id;
      unit[i] = sys[i].unit;
    }
    check(h_, idpd_upload_state(h_, 0, n, pos.data(), vel.data(), acc.data(), id.data(),
                                prop.data(), amp.data(), unit.data()),
          "idpd_upload_state");
    n_ = n;
    uploaded_ = true;
  }

  // Positions, velocities and accelerations of the host rows to the device
  // (the rows the device already holds, in the same order).
  template <class Tpsys>
  void push(const Tpsys& sys) {
    const int n = (int)sys.getNumberOfParticleLocal();
    if (!uploaded_ || n != n_) {
      upload(sys);
      return;
    }
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), acc(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
      put3(&pos[3 * (size_t)i], sys[i].pos);
      put3(&vel[3 * (size_t)i], sys[i].vel);
      put3(&acc[3 * (size_t)i], sys[i].acc);
    }
    check(h_, idpd_set_dynamics(h_, 0, pos.data(), vel.data(), acc.data()), "idpd_set_dynamics");
  }

  // The device rows back into the host system (pos, vel, acc; optionally the
  // per-particle outputs of the passes).
  template <class Tpsys>
  void pull(Tpsys& sys, bool density, bool press, bool nei_cm, bool dsr) {
    const int n = (int)sys.getNumberOfParticleLocal();
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), acc(3 * (size_t)n);
    check(h_, idpd_download_state(h_, 0, pos.data(), vel.data(), acc.data(), nullptr, nullptr,
                                  nullptr, nullptr),
          "idpd_download_state");
    for (int i = 0; i < n; i++) {
      get3(sys[i].pos, &pos[3 * (size_t)i]);
      get3(sys[i].vel, &vel[3 * (size_t)i]);
      get3(sys[i].acc, &acc[3 * (size_t)i]);
    }
    if (!(density || press || nei_cm || dsr)) return;
    std::vector<double> d(density ? 3 * (size_t)n : 0), pr(press ? 3 * (size_t)n : 0),
        cm(nei_cm ? 6 * (size_t)n : 0), ds(dsr ? 3 * (size_t)n : 0);
    check(h_, idpd_download_aux(h_, 0, density ? d.data() : nullptr, press ? pr.data() : nullptr,
                                nei_cm ? cm.data() : nullptr, dsr ? ds.data() : nullptr),
          "idpd_download_aux");
    for (int i = 0; i < n; i++) {
      if (density)
        for (int k = 0; k < 3; k++) sys[i].density[k] = d[3 * (size_t)i + k];
      if (press) get3(sys[i].press, &pr[3 * (size_t)i]);
      if (nei_cm) {
        get3(sys[i].nei_cm_pos[0], &cm[6 * (size_t)i]);
        get3(sys[i].nei_cm_pos[1], &cm[6 * (size_t)i + 3]);
      }
      if (dsr) get3(sys[i].delta_sumr, &ds[3 * (size_t)i]);
    }
  }

  // Parameter::time to the device before a pass that reads it.
  void sync_time() {
    if (!time_ || p_.time == *time_) return;
    p_.time = *time_;
    check(h_, idpd_set_params(h_, 0, &p_), "idpd_set_params");
  }

  int num_particles() const { return n_; }
  void grew(int n) { n_ = n; }

 private:
  template <class V>
  static void put3(double* out, const V& v) {
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
  }
  template <class V>
  static void get3(V& v, const double* in) {
    v.x = in[0];
    v.y = in[1];
    v.z = in[2];
  }

  idpd_params p_;
  const uint32_t* time_;
  idpd_handle* h_ = nullptr;
  int n_ = 0;
  bool uploaded_ = false;
};

namespace detail {
inline std::map<const void*, Session*>& registry() {
  static std::map<const void*, Session*> r;
  return r;
}
inline std::mutex& registry_mutex() {
  static std::mutex m;
  return m;
}
template <class Tpsys>
Session& session_of(const Tpsys& sys) {
  std::lock_guard<std::mutex> lock(registry_mutex());
  auto it = registry().find(&sys);
  if (it == registry().end()) {
    std::fprintf(stderr, "idpd: particle system not bound to a Session (idpd::bind)\n");
    std::abort();
  }
  return *it->second;
}
}  // namespace detail

// Ties a particle system to a session and uploads its rows.
template <class Tpsys>
void bind(Tpsys& sys, Session& s) {
  {
    std::lock_guard<std::mutex> lock(detail::registry_mutex());
    detail::registry()[&sys] = &s;
  }
  s.upload(sys);
}

template <class Tpsys>
void unbind(const Tpsys& sys) {
  std::lock_guard<std::mutex> lock(detail::registry_mutex());
  detail::registry().erase(&sys);
}

// ---------------------------------------------------------------- passes
struct CalcDensity {};
struct CalcForceEpEpDPD {};

// dens_tree.calcForceAllAndWriteBack(CalcDensity(), sys, dinfo): density[3]
// and nei_cm_pos written back (ptcl_class.hpp:53-57).
template <class Tpsys>
void calcForceAllAndWriteBack(CalcDensity, Tpsys& sys) {
  Session& s = detail::session_of(sys);
  s.push(sys);
  check(s.handle(), idpd_density(s.handle()), "idpd_density");
  s.pull(sys, true, false, true, false);
}

// force_tree.calcForceAllAndWriteBack(CalcForceEpEpDPD(), sys, dinfo): acc
// overwritten, press written (ptcl_class.hpp:48-51). Runs on the device state
// of the last CalcDensity pass (the reference's loop changes nothing in
// between, src/main.cpp:173-174).
template <class Tpsys>
void calcForceAllAndWriteBack(CalcForceEpEpDPD, Tpsys& sys) {
  Session& s = detail::session_of(sys);
  s.sync_time();
  check(s.handle(), idpd_force(s.handle()), "idpd_force");
  s.pull(sys, false, true, false, false);
}

template <class Tpsys, class Vec>
void drift_and_predict(Tpsys& sys, double dt, const Vec& box, const Vec& ibox) {
  (void)dt;  // dt and the box are the session's parameters
  (void)box;
  (void)ibox;
  Session& s = detail::session_of(sys);
  s.push(sys);
  check(s.handle(), idpd_drift(s.handle()), "idpd_drift");
  s.pull(sys, false, false, false, true);
}

template <class Tpsys>
void kick(Tpsys& sys, double dt) {
  (void)dt;
  Session& s = detail::session_of(sys);
  s.push(sys);
  check(s.handle(), idpd_kick(s.handle()), "idpd_kick");
  s.pull(sys, false, false, false, false);
}

template <class Tpsys>
void remove_cmdrift_global(Tpsys& sys) {
  Session& s = detail::session_of(sys);
  s.push(sys);
  check(s.handle(), idpd_remove_cmdrift(s.handle()), "idpd_remove_cmdrift");
  s.pull(sys, false, false, false, false);
}

// ForceBonded (bdf_calculator.hpp:11-243), single-node form.
template <class Tpsys>
class ForceBonded {
 public:
  ForceBonded(Tpsys& sys, uint32_t buf_size, uint32_t amp_num,
              const std::vector<uint32_t>& core_amp_id)
      : amp_num_(amp_num) {
    glob_topol_.reserve(buf_size);
    Session& s = detail::session_of(sys);
    s.push(sys);
    check(s.handle(),
          idpd_build_topology(s.handle(), 0, (int32_t)amp_num, (int32_t)core_amp_id.size(),
                              core_amp_id.empty() ? nullptr : core_amp_id.data()),
          "idpd_build_topology");
    MakeGlobalBondedList(sys);
  }

  // acc += bond and bend forces; vir = their virial (bonded_vir).
  template <class Vec>
  void CalcListedForce(Tpsys& sys, Vec& vir) {
    Session& s = detail::session_of(sys);
    s.push(sys);
    double v[3];
    check(s.handle(), idpd_bonded(s.handle(), v), "idpd_bonded");
    s.pull(sys, false, false, false, false);
    vir.x = v[0];
    vir.y = v[1];
    vir.z = v[2];
  }

  const std::vector<uint32_t>& glob_topol() const { return glob_topol_; }
  void ExpandTopolBuffer(uint32_t n) { glob_topol_.reserve(n); }

  // Molecules added by the reaction are bonded from their creation on.
  void AppendMolecules(Tpsys& sys, uint32_t amp_num) {
    amp_num_ = amp_num;
    MakeGlobalBondedList(sys);
  }

 private:
  // glob_topol[4 amp + unit] = row (MakeGlobalBondedList, bdf_calculator.hpp:61-88)
  void MakeGlobalBondedList(const Tpsys& sys) {
    glob_topol_.assign(4 * (size_t)amp_num_, 0xffffffffu);
    const int n = (int)sys.getNumberOfParticleLocal();
    for (int i = 0; i < n; i++)
      if (sys[i].amp_id != 0xffffffffu && sys[i].amp_id < amp_num_ && sys[i].unit < 4u)
        glob_topol_[4 * (size_t)sys[i].amp_id + sys[i].unit] = (uint32_t)i;
  }

  uint32_t amp_num_;
  std::vector<uint32_t> glob_topol_;
};

// ChemManager (chemmanager.hpp:3-282), single-node LOCAL_CHEM_EVENT form.
template <class FP>
class ChemManager {
 public:
  explicit ChemManager(uint32_t seed, int32_t reserve_amp = 4096)
      : seed_(seed), reserve_(reserve_amp) {}

  // New particles are appended to sys (AddNewParticle) and to glob_topol;
  // param.amp_num grows; false when amp_num reached max_amp_num.
  template <class Tpsys, class Topol, class Param>
  bool RandomChemEvent(Tpsys& sys, Topol& glob_topol, Param& param) {
    Session& s = detail::session_of(sys);
    s.push(sys);
    if (!configured_) {
      idpd_chem_config c = {};
      c.p.p_thresld = param.p_thresld;
      c.p.eps = param.eps;
      c.p.influ_rad = param.influ_rad;
      c.p.influ_hei = param.influ_hei;
      c.p.influ_dep = param.influ_dep;
      c.p.influ_grd = param.influ_grd;
      c.p.amp_num = param.amp_num;
      c.p.max_amp_num = param.max_amp_num;
      c.mt_seed = seed_;
      c.beg_chem = 0xffffffffu;  // events only through this call
      c.n_core = (int32_t)param.core_ptcl_id.size();
      if (c.n_core > IDPD_CHEM_MAX_CORE) {
        std::fprintf(stderr, "idpd: at most %d core particles\n", IDPD_CHEM_MAX_CORE);
        std::abort();
      }
      for (int k = 0; k < c.n_core; k++) c.core_ptcl_id[k] = param.core_ptcl_id[k];
      c.reserve_amp = reserve_;
      check(s.handle(), idpd_set_chem(s.handle(), 0, &c), "idpd_set_chem");
      configured_ = true;
    }
    int32_t cont = 1;
    check(s.handle(), idpd_chem_event(s.handle(), &cont), "idpd_chem_event");
    int32_t n = 0;
    check(s.handle(), idpd_num_particles(s.handle(), 0, &n), "idpd_num_particles");
    const int n0 = (int)sys.getNumberOfParticleLocal();
    if (n > n0) {
      std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n);
      std::vector<uint32_t> id(n), prop(n), amp(n), unit(n);
      check(s.handle(), idpd_download_state(s.handle(), 0, pos.data(), vel.data(), nullptr,
                                            id.data(), prop.data(), amp.data(), unit.data()),
            "idpd_download_state");
      for (int i = n0; i < n; i++) {
        FP p = FP();
        p.pos.x = pos[3 * (size_t)i];
        p.pos.y = pos[3 * (size_t)i + 1];
        p.pos.z = pos[3 * (size_t)i + 2];
        p.vel.x = vel[3 * (size_t)i];
        p.vel.y = vel[3 * (size_t)i + 1];
        p.vel.z = vel[3 * (size_t)i + 2];
        p.id = id[i];
        p.prop = prop[i];
        p.amp_id = amp[i];
        p.unit = unit[i];
        sys.AddNewParticle(p);
        glob_topol.push_back((uint32_t)i);  // rows of each new molecule, unit order
      }
      s.grew(n);
    }
    idpd_chem_info info;
    check(s.handle(), idpd_chem_get_info(s.handle(), 0, &info, nullptr, 0), "idpd_chem_get_info");
    param.amp_num = info.amp_num;
    h2t_.resize(info.n_core);
    core_h_.resize(info.n_core);
    for (int k = 0; k < info.n_core; k++) {
      h2t_[k] = Vec3{info.h2t[k][0], info.h2t[k][1], info.h2t[k][2]};
      core_h_[k] = Vec3{info.core_h[k][0], info.core_h[k][1], info.core_h[k][2]};
    }
    return cont != 0;
  }

  // Per core particle, the unit head-to-tail vector (membrane normal) and the
  // projected core position of the last event (chemmanager.hpp:123-135,
  // 183-189), the arrays Observer::MembNormalVect reads (observer.hpp:276);
  // empty before the first event. The reference declares both arrays but
  // never fills them.
  struct Vec3 {
    double x, y, z;
  };
  const std::vector<Vec3>& h2t_vecs() const { return h2t_; }
  const std::vector<Vec3>& core_poss_h() const { return core_h_; }

 private:
  uint32_t seed_;
  int32_t reserve_;
  bool configured_ = false;
  std::vector<Vec3> h2t_, core_h_;
};

}  // namespace idpd
