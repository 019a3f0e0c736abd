// Host side of the C ABI in include/idpd_engine.h: handle life cycle,
// replica layout, uploads and downloads, the per-step launch sequence and its
// CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "idpd_engine.h"
#include "state.cuh"

using namespace idpd;

namespace {

// The message of the last failure without a handle, per host thread (calls
// on different handles may run on different threads).
thread_local std::string g_lib_err;

struct Staged {  // one replica's rows as uploaded (upload order)
  std::vector<double> pos, vel, acc;
  std::vector<uint32_t> id, prop, amp_id, unit;
  std::vector<uint32_t> topol;  // local rows, 4 per molecule
  std::vector<float> cf_bend;
  int n_amp = 0;
};

}  // namespace

namespace idpd {
void set_library_error(const char* msg) { g_lib_err = msg; }
}  // namespace idpd

struct idpd_handle {
  int device = 0;
  int flags = 0;
  int sort_period = 100;
  int R = 1;
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<idpd_params> params;
  std::vector<char> params_set;
  std::vector<Staged> staged;
  std::vector<int> n;       // rows per replica
  std::vector<int> n_amp;   // molecules per replica
  std::vector<RepDev> reps_h;
  bool layout_dirty = true;   // device arrays must be rebuilt from staging
  bool reps_dirty = true;     // RepDev table must be re-uploaded
  bool on_device = false;     // device arrays hold the current state
  bool density_valid = false;
  int cap = 0;                // allocated rows
  int ncell_cap = 0, ncell_tot = 0;
  int nblk = 0, nblk_cap = 0;
  int n_tot = 0, n_amp_tot = 0, n_amp_cap = 0;
  DevState d{}, o{};          // state and reorder scratch
  std::vector<void*> allocs;
  // aux buffers of the fine-grained API
  double *press64 = nullptr, *cm64 = nullptr, *vir_part = nullptr;
  double* xfer = nullptr;     // device staging of the per-step exchange
  uint32_t* cm_cnt = nullptr;
  int* amp_rep = nullptr;
  // graph
  cudaGraphExec_t graph = nullptr;
  int steps_since_sort = 0;
  float last_ms = 0.f;
  PairTuning tune{1, 0.0f, 16, 1, 32};
  bool vl_dirty = true;                 // cells rebuilt outside the step: the kept lists are stale
  std::string err;
  // chemistry (replica 0 of a one-replica handle)
  bool chem_on = false;
  // precursor conversion, per replica
  std::vector<idpd_precursor> prec;
  bool prec_any = false;
  unsigned long long* prec_dev = nullptr;  // [R] conversions
  idpd_chem_config chem_cfg{};
  ChemDev* chem = nullptr;        // device, kept across re-layouts (MT state)
  ChemBuffers chem_buf{};         // scratch, sized with the layout
  int chem_amp_cap = 0;           // molecule slots of the layout (with reserve)
  int* chem_flag_host = nullptr;  // pinned: the device's stopped flag
  size_t chem_buf_total = 0, chem_buf_tcap = 0;  // sizes of the allocated scratch
  bool chem_stopped = false;
  // observation (Observer) every obs_period steps
  int obs_period = 0, obs_cap = 0;
  idpd_observation* obs_rec = nullptr;  // device records, kept across re-layouts
  int* obs_count = nullptr;
  ObsBuffers obs_buf{};                 // per-layout scratch (null until needed)
  cudaGraphExec_t graph_obs = nullptr;  // the step with the observation
  // K steps in one launch: the step inside a WHILE conditional node
  cudaGraphExec_t graph_loop = nullptr;
  cudaStream_t cst = nullptr;  // captures the bodies of the step's IF nodes
  int* loop_left = nullptr;  // device count of the loop's steps left
  bool loop_failed = false;  // the loop graph could not be built: one launch per step
  WalkState* walks = nullptr;           // FDPS multi-walk buffers (created on first use)
  unsigned long long* pair_sum = nullptr;  // device word of idpd_pair_count
  // asynchronous trajectory frames (idpd_dump_xyz_async): device staging in
  // upload order, its pinned host copy, the copy stream and the writer thread
  cudaStream_t dump_st = nullptr;
  // idpd_step_host and idpd_download_state: the copy stream of the host
  // exchange and its events
  cudaStream_t xst = nullptr;
  cudaEvent_t x_drift = nullptr, x_done = nullptr, x_mid = nullptr;
  cudaEvent_t dump_ready = nullptr, dump_done = nullptr;
  unsigned char* dump_dev = nullptr;
  unsigned char* dump_host = nullptr;
  size_t dump_cap = 0;
  std::thread dump_thread;
  int dump_rc = IDPD_OK;        // first failed frame's status (read by idpd_dump_wait)
  std::string dump_msg;
  bool pairs_valid = false;             // a density pass has run on the current layout
};

namespace {

int fail(idpd_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h)
    h->err = buf;
  else
    g_lib_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(h, IDPD_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));      \
  } while (0)

template <class T>
int dalloc(idpd_handle* h, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return fail(h, IDPD_ERR_CUDA, "cudaMalloc(%zu B): %s", count * sizeof(T),
                                    cudaGetErrorString(e));
  h->allocs.push_back((void*)*p);
  return IDPD_OK;
}

void free_all(idpd_handle* h) {
  if (h->graph_loop) {
    cudaGraphExecDestroy(h->graph_loop);
    h->graph_loop = nullptr;
  }
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (h->graph_obs) {
    cudaGraphExecDestroy(h->graph_obs);
    h->graph_obs = nullptr;
  }
  h->obs_buf.part = nullptr;
  h->obs_buf.mvir = h->obs_buf.mdif = nullptr;
  for (void* p : h->allocs) cudaFree(p);
  h->allocs.clear();
  h->d = DevState{};
  h->o = DevState{};
  h->press64 = h->cm64 = h->vir_part = nullptr;
  h->xfer = nullptr;
  h->cm_cnt = nullptr;
  h->amp_rep = nullptr;
  h->chem_buf = ChemBuffers{h->chem, nullptr, nullptr, nullptr, nullptr};
  h->chem_buf_total = h->chem_buf_tcap = 0;
  h->cap = h->ncell_cap = h->nblk_cap = h->n_amp_cap = 0;
}

void invalidate_graph(idpd_handle* h) {
  if (h->graph_loop) {
    cudaGraphExecDestroy(h->graph_loop);
    h->graph_loop = nullptr;
  }
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  if (h->graph_obs) {
    cudaGraphExecDestroy(h->graph_obs);
    h->graph_obs = nullptr;
  }
}

int check_params(idpd_handle* h, const idpd_params* p) {
  for (int k = 0; k < 3; k++) {
    if (!(std::isfinite(p->box[k]) && p->box[k] >= 3.0))
      return fail(h, IDPD_ERR_INVALID_ARG, "box[%d] = %g: every box side must be >= 3 (3 cells of the cutoff 1)", k, p->box[k]);
  }
  if (!(std::isfinite(p->dt) && p->dt > 0.0)) return fail(h, IDPD_ERR_INVALID_ARG, "dt must be > 0");
  if (p->form < IDPD_FORM_MDPD || p->form > IDPD_FORM_WARREN)
    return fail(h, IDPD_ERR_INVALID_ARG, "unknown form %d", p->form);
  if (p->form == IDPD_FORM_WARREN && !(p->warren_rd > 0.0 && p->warren_rd <= 1.0))
    return fail(h, IDPD_ERR_INVALID_ARG, "warren_rd must be in (0, 1]");
  const double* tabs[4] = {&p->cf_c[0][0], &p->cf_g[0][0], &p->cf_r[0][0], &p->cf_m[0][0][0]};
  const int sz[4] = {9, 9, 9, 27};
  for (int t = 0; t < 4; t++)
    for (int k = 0; k < sz[t]; k++)
      if (!std::isfinite(tabs[t][k])) return fail(h, IDPD_ERR_NONFINITE, "non-finite coefficient table entry");
  return IDPD_OK;
}

// Frame cells have side >= the cutoff (nf = floor(box)); the search grid
// splits each frame cell into `reach` cells per axis. Positions are stored
// relative to frame cells, so the search grid never changes a pair term.
void fill_repdev(RepDev& R, const idpd_params& p, int reach, float skin) {
  const double cut = 1.0 + (double)skin;  // frame cells: the cutoff plus the skin
  R.reach = reach;
  R.rshift = reach == 2 ? 1 : 0;
  for (int k = 0; k < 3; k++) {
    R.box[k] = p.box[k];
    R.ibox[k] = 1.0 / p.box[k];
    R.nf[k] = (int)(p.box[k] / cut);
    R.nc[k] = R.nf[k] * reach;
    R.inv_cs[k] = (double)R.nc[k] / p.box[k];
    R.cs[k] = p.box[k] / (double)R.nf[k];
    R.cs_f[k] = (float)R.cs[k];
    R.cs_lo[k] = (float)(R.cs[k] - (double)R.cs_f[k]);
  }
  R.ncell = R.nc[0] * R.nc[1] * R.nc[2];
  R.dt = p.dt;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R.cf_c[3 * i + j] = (float)p.cf_c[i][j];
      R.cf_g[3 * i + j] = (float)p.cf_g[i][j];
      R.cf_r[3 * i + j] = (float)p.cf_r[i][j];
      for (int k = 0; k < 3; k++) R.cf_m[9 * i + 3 * j + k] = (float)p.cf_m[i][j][k];
    }
  R.wa = (float)p.warren_a;
  R.wb = (float)p.warren_b;
  R.wrd = p.form == IDPD_FORM_WARREN ? (float)p.warren_rd : 1.0f;
  R.winv_rd = 1.0f / R.wrd;
  const double rd = p.form == IDPD_FORM_WARREN ? p.warren_rd : 1.0;
  R.wnorm = (float)(15.0 / (2.0 * 3.14159265358979323846 * rd * rd * rd));
  R.cf_s = (float)p.cf_s;
  R.seed = p.seed;
  R.form = p.form;
  // density weights reach (1-r)^2 <= 1, or wnorm (1 - r/rd)^2 <= wnorm (Warren)
  int k = 0;
  const double wmax = p.form == IDPD_FORM_WARREN ? (double)R.wnorm : 1.0;
  while (std::ldexp(1.0, k) < wmax) k++;
  R.dens_prescale = (float)std::ldexp(1.0, -k);
  R.dens_unscale = std::ldexp(1.0, k - 23);
  R.dens_unscale_f = (float)R.dens_unscale;
}

// A caller buffer that lives in device or managed memory, which the kernels
// read or write where it lies; null for host memory, which goes through the
// staging buffer and a copy engine (page-locked memory read by the kernels
// over the host link measured slower than the copies).
const void* device_view(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return p;
  return nullptr;
}

// Bit f set when some replica uses pair-force form f.
int form_mask(const idpd_handle* h) {
  int m = 0;
  for (int r = 0; r < h->R; r++) m |= 1 << h->params[r].form;
  return m;
}

// fill_repdev plus the replica's precursor conversion.
void fill_rep(const idpd_handle* h, int r, RepDev& R) {
  fill_repdev(R, h->params[r], h->tune.reach, h->tune.skin);
  const idpd_precursor& q = h->prec[r];
  R.prec_on = q.enabled ? 1 : 0;
  R.prec_from = q.prop_from;
  R.prec_near = q.prop_near;
  R.prec_to = q.prop_to;
  R.prec_thr = q.threshold;
  R.prec_seed = q.seed;
}

// Allocates (or grows) every device array for the current layout.
int ensure_capacity(idpd_handle* h, int rows, int ncell, int nblk, int namp) {
  const bool grow = rows > h->cap || ncell > h->ncell_cap || nblk > h->nblk_cap ||
                    namp > h->n_amp_cap;
  if (!grow && h->d.px) return IDPD_OK;
  free_all(h);
  const int cap = std::max(rows, 1);
  const int cc = std::max(ncell, 1);
  const int bc = std::max(nblk, 1);
  const int ac = std::max(namp, 1);
  DevState& d = h->d;
  DevState& o = h->o;
  int rc = IDPD_OK;
#define AL(ptr, cnt) \
  if ((rc = dalloc(h, &(ptr), (cnt))) != IDPD_OK) return rc
  for (DevState* s : {&d, &o}) {
    AL(s->px, cap); AL(s->py, cap); AL(s->pz, cap);
    AL(s->vx, cap); AL(s->vy, cap); AL(s->vz, cap);
    AL(s->ax, cap); AL(s->ay, cap); AL(s->az, cap);
    AL(s->dsx, cap); AL(s->dsy, cap); AL(s->dsz, cap);
    AL(s->id, cap); AL(s->prop, cap); AL(s->amp_id, cap); AL(s->unit, cap);
    AL(s->orig, cap); AL(s->key, cap);
  }
  AL(d.loc, cap);
  AL(h->xfer, 9 * (size_t)cap);
  AL(d.slot, cap);
  AL(d.cell_cnt, cc);
  AL(d.cell_start, cc + 1);
  AL(d.scan_part, (cc + 4095) / 4096 + 1);
  AL(d.perm, cap); AL(d.rank, cap); AL(d.scell, cap);
  AL(d.posf, cap); AL(d.velf, cap); AL(d.densf, cap); AL(d.poslo, cap);
  AL(d.fq, 4 * (size_t)cap);
  AL(d.nbl, (size_t)kNbrCap * cap); AL(d.nbn, cap);
  AL(d.dsum, 4 * (size_t)cap);
  AL(d.topol, 4 * ac);
  AL(d.cf_bend, ac);
  AL(d.reps, h->R);
  AL(d.tab64, h->R);
  AL(d.rep_time, h->R);
  AL(d.blk_rep, bc);
  AL(d.blk_row, bc);
  AL(d.blk_part, 3 * bc);
  AL(d.npair, cap);
  AL(h->pair_sum, 1);
  AL(h->loop_left, 1);
  AL(d.rep_mean, 3 * h->R);
  AL(d.err, 1);
  AL(h->amp_rep, ac);
  if (h->flags & (IDPD_CFG_FP64_PAIRS | IDPD_CFG_FP64_KEPT)) { AL(d.dens64, 3 * (size_t)cap); }
  if (h->flags & IDPD_CFG_FP64_KEPT) { AL(d.svel, 4 * (size_t)cap); }
#undef AL
  d.pq = nullptr;
  d.dqx = d.dqy = d.dqz = nullptr;
  CK(cudaMemsetAsync(d.cell_cnt, 0, sizeof(int) * cc, h->st));
  CK(cudaMemsetAsync(d.err, 0, sizeof(int), h->st));
  CK(cudaMemsetAsync(d.dsum, 0, sizeof(unsigned long long) * 4 * (size_t)cap, h->st));
  CK(cudaMemsetAsync(d.npair, 0, sizeof(uint32_t) * (size_t)cap, h->st));
  h->cap = cap;
  h->ncell_cap = cc;
  h->nblk_cap = bc;
  h->n_amp_cap = ac;
  return IDPD_OK;
}

// Per-particle virial of the pair pass (fine-grained API and observation).
int ensure_press(idpd_handle* h) {
  if (h->d.pq) return IDPD_OK;
  int rc;
  DevState& d = h->d;
  if ((rc = dalloc(h, &d.pq, 4 * (size_t)h->cap))) return rc;
  invalidate_graph(h);
  return IDPD_OK;
}

// Scratch of the observation for the current layout.
int ensure_obs(idpd_handle* h) {
  int rc = ensure_press(h);
  if (rc) return rc;
  ObsBuffers& b = h->obs_buf;
  if (!b.part) {
    if ((rc = dalloc(h, &b.part, (size_t)h->nblk_cap)) ||
        (rc = dalloc(h, &b.mvir, 3 * (size_t)h->n_amp_cap)) ||
        (rc = dalloc(h, &b.mdif, (size_t)h->n_amp_cap)))
      return rc;
    invalidate_graph(h);
  }
  b.rec = h->obs_rec;
  b.count = h->obs_count;
  b.cap = h->obs_cap;
  b.period = h->obs_period;
  return IDPD_OK;
}

// Kept neighbour lists (skin > 0): buffers and the rebuild record, which
// starts with a forced rebuild.
int ensure_verlet(idpd_handle* h) {
  if (h->tune.skin <= 0.0f) return IDPD_OK;
  DevState& d = h->d;
  if (!d.vl) {
    int rc;
    if ((rc = dalloc(h, &d.vl, (size_t)kVerletCap * h->cap)) || (rc = dalloc(h, &d.vn, h->cap)) ||
        (rc = dalloc(h, &d.okey, h->cap)) ||
        (rc = dalloc(h, &d.drx, h->cap)) || (rc = dalloc(h, &d.dry, h->cap)) ||
        (rc = dalloc(h, &d.drz, h->cap)) || (rc = dalloc(h, &d.vdev, 1)))
      return rc;
  }
  VerletDev v{};
  const double skin = h->tune.skin;
  const double half = 0.5 * skin - 1.0e-5;  // margin for the float displacement test
  v.thr2 = (float)(half * half);
  v.rv2 = (float)((1.0 + skin) * (1.0 + skin) + 1.0e-4);
  v.force = 1;
  CK(cudaMemcpyAsync(d.vdev, &v, sizeof(v), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->vl_dirty = false;
  invalidate_graph(h);
  return IDPD_OK;
}

// The precursor marks of pass 1 (read by the conversion kernel).
int ensure_phit(idpd_handle* h) {
  if (!h->prec_any || h->d.phit) return IDPD_OK;
  int rc = dalloc(h, &h->d.phit, h->cap);
  if (rc) return rc;
  invalidate_graph(h);
  return IDPD_OK;
}

// Buffers of the kept lists for the current layout, and a forced rebuild
// when cells were rebuilt outside the step.
int ensure_verlet_ready(idpd_handle* h) {
  if (h->tune.skin <= 0.0f) return IDPD_OK;
  if (!h->d.vl) return ensure_verlet(h);
  if (h->vl_dirty) {
    static const int kOne = 1;
    CK(cudaMemcpyAsync(&h->d.vdev->force, &kOne, sizeof(int), cudaMemcpyHostToDevice, h->st));
    h->vl_dirty = false;
  }
  return IDPD_OK;
}

int ensure_aux(idpd_handle* h) {
  if (h->press64) return IDPD_OK;
  int rc = ensure_press(h);
  if (rc) return rc;
  DevState& d = h->d;
  if ((rc = dalloc(h, &d.dqx, h->cap)) ||
      (rc = dalloc(h, &d.dqy, h->cap)) || (rc = dalloc(h, &d.dqz, h->cap)) ||
      (rc = dalloc(h, &h->press64, 3 * (size_t)h->cap)) ||
      (rc = dalloc(h, &h->cm64, 6 * (size_t)h->cap)) ||
      (rc = dalloc(h, &h->cm_cnt, 2 * (size_t)h->cap)) ||
      (rc = dalloc(h, &h->vir_part, 3 * (size_t)h->n_amp_cap)))
    return rc;
  invalidate_graph(h);  // DevState changed (aux pointers)
  return IDPD_OK;
}

// Pulls the device state of every replica back into the staging buffers
// (upload order) so that the layout can be rebuilt.
int pull_to_staging(idpd_handle* h);

// Scratch of the reaction event for the current layout, and the layout's
// capacities in the device record (its MT state is kept).
int chem_layout(idpd_handle* h) {
  const RepDev& R = h->reps_h[0];
  const int amp_cap = R.n_amp + h->chem_cfg.reserve_amp;
  const int tcap = std::max(h->chem_cfg.reserve_amp, 1);
  const int total = std::max(h->chem_cfg.n_core * amp_cap, 1);
  ChemBuffers& b = h->chem_buf;
  b.chem = h->chem;
  int rc = IDPD_OK;
  if ((size_t)total > h->chem_buf_total) {
    if ((rc = dalloc(h, &b.flags, (size_t)total))) return rc;
    if ((rc = dalloc(h, &b.chunk, (size_t)(total + 1023) / 1024))) return rc;
    h->chem_buf_total = (size_t)total;
  }
  if ((size_t)tcap > h->chem_buf_tcap) {
    if ((rc = dalloc(h, &b.targets, 2 * (size_t)tcap))) return rc;
    if ((rc = dalloc(h, &b.draws, 25 * (size_t)tcap))) return rc;
    h->chem_buf_tcap = (size_t)tcap;
  }
  h->chem_amp_cap = amp_cap;
  const int caps[3] = {R.n + 4 * h->chem_cfg.reserve_amp, amp_cap, tcap};
  const uint32_t amp_num = (uint32_t)R.n_amp;
  CK(cudaMemcpyAsync(&h->chem->row_cap, caps, sizeof(caps), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(&h->chem->amp_num, &amp_num, sizeof(uint32_t), cudaMemcpyHostToDevice, h->st));
  std::vector<float> cfb(h->chem_cfg.reserve_amp, (float)h->params[0].cf_b);
  if (!cfb.empty())
    CK(cudaMemcpyAsync(h->d.cf_bend + R.amp_off + R.n_amp, cfb.data(), sizeof(float) * cfb.size(),
                       cudaMemcpyHostToDevice, h->st));
  return IDPD_OK;
}

// Particle and molecule counts of replica 0 after device-side growth.
int sync_counts(idpd_handle* h) {
  if (!h->chem_on || !h->on_device || h->layout_dirty) return IDPD_OK;
  RepDev R;
  CK(cudaMemcpyAsync(&R, h->d.reps, sizeof(RepDev), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->reps_h[0].n = R.n;
  h->reps_h[0].n_amp = R.n_amp;
  h->n[0] = R.n;
  h->n_amp[0] = R.n_amp;
  return IDPD_OK;
}

// Builds the layout from the staging buffers and uploads everything.
int commit(idpd_handle* h) {
  if (!h->layout_dirty && !h->reps_dirty) return IDPD_OK;
  for (int r = 0; r < h->R; r++)
    if (!h->params_set[r]) return fail(h, IDPD_ERR_STATE, "replica %d has no parameters", r);
  if (h->layout_dirty) {
    h->pairs_valid = false;
    invalidate_graph(h);
    h->reps_h.assign(h->R, RepDev{});
    int row = 0, cell = 0, blk = 0, amp = 0;
    std::vector<int> blk_rep, blk_row;
    for (int r = 0; r < h->R; r++) {
      RepDev& R = h->reps_h[r];
      fill_rep(h, r, R);
      // a reaction appends molecules on the device: room for them after the rows
      const int extra_amp = (h->chem_on && r == 0) ? h->chem_cfg.reserve_amp : 0;
      R.row_off = row;
      R.n = h->n[r];
      R.cell_off = cell;
      R.blk_off = blk;
      R.nblk = (R.n + 4 * extra_amp + kRowBlock - 1) / kRowBlock;
      R.n_amp = h->staged[r].n_amp;
      R.amp_off = amp;
      for (int b = 0; b < R.nblk; b++) {
        blk_rep.push_back(r);
        blk_row.push_back(row + b * kRowBlock);
      }
      row += R.n + 4 * extra_amp;
      cell += R.ncell;
      blk += R.nblk;
      amp += R.n_amp + extra_amp;
      if ((long long)row >= (1ll << 25))  // the sorted row of a list entry has 25 bits
        return fail(h, IDPD_ERR_CAPACITY, "more than 2^25 particle rows in one handle");
      if ((long long)cell >= (1ll << 31) - 1) return fail(h, IDPD_ERR_CAPACITY, "too many cells");
    }
    h->n_tot = row;
    h->ncell_tot = cell;
    h->nblk = blk;
    h->n_amp_tot = amp;
    int rc = ensure_capacity(h, row, cell, blk, amp);
    if (rc) return rc;
    DevState& d = h->d;
    CK(cudaMemcpyAsync(d.blk_rep, blk_rep.data(), sizeof(int) * blk, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(d.blk_row, blk_row.data(), sizeof(int) * blk, cudaMemcpyHostToDevice, h->st));
    // rows: host transposes into SoA staging, one copy per field
    std::vector<double> buf(9 * (size_t)std::max(row, 1));
    std::vector<uint32_t> ub(5 * (size_t)std::max(row, 1));
    std::vector<uint32_t> topol(4 * (size_t)std::max(amp, 1), 0u);
    std::vector<float> cfb(std::max(amp, 1), 0.0f);
    std::vector<int> amp_rep(std::max(amp, 1), h->R - 1);
    std::vector<uint32_t> time(h->R);
    for (int r = 0; r < h->R; r++) {
      const Staged& s = h->staged[r];
      const RepDev& R = h->reps_h[r];
      for (int k = 0; k < R.n; k++) {
        const size_t i = (size_t)R.row_off + k;
        for (int c = 0; c < 3; c++) {
          buf[c * (size_t)row + i] = s.pos[3 * (size_t)k + c];
          buf[(3 + c) * (size_t)row + i] = s.vel[3 * (size_t)k + c];
          buf[(6 + c) * (size_t)row + i] = s.acc[3 * (size_t)k + c];
        }
        ub[i] = s.id[k];
        ub[row + i] = s.prop[k];
        ub[2 * (size_t)row + i] = s.amp_id[k];
        ub[3 * (size_t)row + i] = s.unit[k];
        ub[4 * (size_t)row + i] = (uint32_t)i;
      }
      for (int a = 0; a < R.n_amp; a++) {
        for (int u = 0; u < 4; u++)
          topol[4 * (size_t)(R.amp_off + a) + u] = (uint32_t)R.row_off + s.topol[4 * (size_t)a + u];
        cfb[R.amp_off + a] = s.cf_bend[a];
        amp_rep[R.amp_off + a] = r;
      }
      time[r] = h->params[r].time;
    }
    double* dst[9] = {d.px, d.py, d.pz, d.vx, d.vy, d.vz, d.ax, d.ay, d.az};
    for (int c = 0; c < 9; c++)
      CK(cudaMemcpyAsync(dst[c], buf.data() + c * (size_t)row, sizeof(double) * row,
                         cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(d.loc, ub.data() + 4 * (size_t)row, sizeof(uint32_t) * row,
                       cudaMemcpyHostToDevice, h->st));
    uint32_t* udst[5] = {d.id, d.prop, d.amp_id, d.unit, d.orig};
    for (int c = 0; c < 5; c++)
      CK(cudaMemcpyAsync(udst[c], ub.data() + c * (size_t)row, sizeof(uint32_t) * row,
                         cudaMemcpyHostToDevice, h->st));
    CK(cudaMemsetAsync(d.dsx, 0, sizeof(double) * std::max(row, 1), h->st));
    CK(cudaMemsetAsync(d.dsy, 0, sizeof(double) * std::max(row, 1), h->st));
    CK(cudaMemsetAsync(d.dsz, 0, sizeof(double) * std::max(row, 1), h->st));
    if (amp > 0) {
      CK(cudaMemcpyAsync(d.topol, topol.data(), sizeof(uint32_t) * 4 * amp, cudaMemcpyHostToDevice, h->st));
      CK(cudaMemcpyAsync(d.cf_bend, cfb.data(), sizeof(float) * amp, cudaMemcpyHostToDevice, h->st));
      CK(cudaMemcpyAsync(h->amp_rep, amp_rep.data(), sizeof(int) * amp, cudaMemcpyHostToDevice, h->st));
    }
    CK(cudaMemcpyAsync(d.rep_time, time.data(), sizeof(uint32_t) * h->R, cudaMemcpyHostToDevice, h->st));
    if (h->chem_on) {
      int rc2 = chem_layout(h);
      if (rc2) return rc2;
    }
    CK(cudaStreamSynchronize(h->st));
    h->layout_dirty = false;
    h->reps_dirty = true;
    h->on_device = true;
    h->density_valid = false;
    h->steps_since_sort = 0;
  }
  if (h->reps_dirty) {
    for (int r = 0; r < h->R; r++) {
      RepDev& R = h->reps_h[r];
      const RepDev keep = R;
      fill_rep(h, r, R);
      R.row_off = keep.row_off; R.n = keep.n; R.cell_off = keep.cell_off; R.blk_off = keep.blk_off;
      R.nblk = keep.nblk; R.n_amp = keep.n_amp; R.amp_off = keep.amp_off;
      if (R.ncell != keep.ncell) return fail(h, IDPD_ERR_STATE, "box change alters the cell grid; re-upload the state");
    }
    CK(cudaMemcpyAsync(h->d.reps, h->reps_h.data(), sizeof(RepDev) * h->R, cudaMemcpyHostToDevice, h->st));
    std::vector<RepTab64> t64(h->R);
    for (int r = 0; r < h->R; r++) {
      const idpd_params& p = h->params[r];
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          t64[r].cf_c[3 * i + j] = p.cf_c[i][j];
          t64[r].cf_g[3 * i + j] = p.cf_g[i][j];
          t64[r].cf_r[3 * i + j] = p.cf_r[i][j];
          for (int k = 0; k < 3; k++) t64[r].cf_m[9 * i + 3 * j + k] = p.cf_m[i][j][k];
        }
      t64[r].wa = p.warren_a;
      t64[r].wb = p.warren_b;
      t64[r].wrd = p.form == IDPD_FORM_WARREN ? p.warren_rd : 1.0;
    }
    CK(cudaMemcpyAsync(h->d.tab64, t64.data(), sizeof(RepTab64) * h->R, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->reps_dirty = false;
  }
  return IDPD_OK;
}

// (Re)allocates only the cell arrays, keeping the particle arrays.
int realloc_cells(idpd_handle* h, int ncell) {
  DevState& d = h->d;
  if (ncell > h->ncell_cap) {
    for (void* p : {(void*)d.cell_cnt, (void*)d.cell_start, (void*)d.scan_part}) {
      h->allocs.erase(std::remove(h->allocs.begin(), h->allocs.end(), p), h->allocs.end());
      cudaFree(p);
    }
    int rc;
    if ((rc = dalloc(h, &d.cell_cnt, ncell)) || (rc = dalloc(h, &d.cell_start, ncell + 1)) ||
        (rc = dalloc(h, &d.scan_part, (ncell + 4095) / 4096 + 1)))
      return rc;
    h->ncell_cap = ncell;
  }
  CK(cudaMemsetAsync(d.cell_cnt, 0, sizeof(int) * h->ncell_cap, h->st));
  return IDPD_OK;
}

// Applies a new cell reach to a committed layout: new cell grids and cell
// offsets, same particle rows.
int retune_cells(idpd_handle* h) {
  invalidate_graph(h);
  int cell = 0;
  for (int r = 0; r < h->R; r++) {
    RepDev& R = h->reps_h[r];
    const RepDev keep = R;
    fill_rep(h, r, R);
    R.row_off = keep.row_off; R.n = keep.n; R.blk_off = keep.blk_off; R.nblk = keep.nblk;
    R.n_amp = keep.n_amp; R.amp_off = keep.amp_off;
    R.cell_off = cell;
    cell += R.ncell;
  }
  h->ncell_tot = cell;
  int rc = realloc_cells(h, cell);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->d.reps, h->reps_h.data(), sizeof(RepDev) * h->R, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->density_valid = false;
  return IDPD_OK;
}

int check_device_error(idpd_handle* h) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, h->d.err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  if (e == 0) return IDPD_OK;
  CK(cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
  switch (e) {
    case kErrNonFinite: return fail(h, IDPD_ERR_NONFINITE, "non-finite pair force");
    case kErrComBox: return fail(h, IDPD_ERR_INVALID_ARG, "neighbour centre of mass needs >= 5 cells per axis (box >= 5)");
    case kErrChemCapacity: return fail(h, IDPD_ERR_CAPACITY, "reaction event exceeds the reserved molecules (idpd_chem_config.reserve_amp)");
    case kErrDensPairs: return fail(h, IDPD_ERR_CAPACITY, "more than %d pairs within the cutoff of one particle", kDensPairsMax);
    default: return fail(h, IDPD_ERR_STATE, "device error code %d", e);
  }
}

// Arithmetic of the pair passes chosen at creation.
int pair_mode(const idpd_handle* h) {
  if (h->flags & IDPD_CFG_FP64_PAIRS) return kPairsF64;
  if (h->flags & IDPD_CFG_FP64_KEPT) return kPairsF64Kept;
  return kPairsF32;
}

// Cell list over the current positions (no drift).
void enqueue_cells(idpd_handle* h, bool drift) {
  h->vl_dirty = true;
  launch_drift_bin(h->d, h->nblk, drift, h->st);
  launch_scan(h->d, h->ncell_tot, h->R - 1, h->st);
  launch_scatter_sort_pack(h->d, h->nblk, h->ncell_tot, true, h->st);
}

// Work that most steps skip goes, in a captured step, into the body of an IF
// node: begin_if adds the node after the kernel that sets its condition
// (cond launches it) and starts capturing the body on h->cst; the caller
// enqueues the work on the returned stream; end_if ends the body. When the
// stream is not capturing (a step enqueued directly), the work goes to h->st
// and its kernels skip themselves, as they do inside the body too.
struct IfScope {
  cudaStream_t st;
  bool body;
};
template <class Cond>
IfScope begin_if(idpd_handle* h, Cond&& cond) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  const cudaGraphEdgeData* edges = nullptr;
  size_t nd = 0;
  if ((h->flags & IDPD_CFG_PLAIN_GRAPHS) ||
      cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, &edges, &nd) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return {h->st, false};
  cudaGraphConditionalHandle ch;
  if (cudaGraphConditionalHandleCreate(&ch, g, 0, cudaGraphCondAssignDefault) != cudaSuccess)
    return {h->st, false};
  cond(ch);
  if (cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, &edges, &nd) != cudaSuccess)
    return {h->st, false};
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = ch;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, deps, edges, nd, &cp) != cudaSuccess) return {h->st, false};
  cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (cudaStreamBeginCaptureToGraph(h->cst, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return {h->st, false};  // an empty body: the kernels follow on h->st
  return {h->cst, true};
}

void end_if(idpd_handle* h, const IfScope& s) {
  if (!s.body) return;
  cudaGraph_t body;
  cudaStreamEndCapture(h->cst, &body);
}

// One MD step; `observe` adds the per-particle virial to the pair pass and
// the observation kernels (the records are written only for replicas whose
// step counter is due).
void enqueue_step(idpd_handle* h, bool observe, cudaEvent_t drift_done = nullptr) {
  const int mode = pair_mode(h);
  DevState d = h->d;  // the step writes no fine-grained side outputs
  d.dqx = d.dqy = d.dqz = nullptr;
  const bool verlet = d.vdev && h->tune.skin > 0.0f && mode != kPairsF64;
  if (verlet) {  // cells and lists only on rebuild steps
    const int* gate = &d.vdev->rebuild;
    launch_drift_disp(d, h->nblk, h->st);
    if (drift_done) cudaEventRecord(drift_done, h->st);  // positions final
    launch_vl_decide(d, h->st);
    const auto rebuild = [&](cudaGraphConditionalHandle c) { launch_cond_flag(c, gate, h->st); };
    IfScope c = begin_if(h, rebuild);
    launch_bin_gated(d, h->nblk, c.st);
    launch_scan(d, h->ncell_tot, h->R - 1, c.st, gate);
    launch_scatter_sort(d, h->nblk, h->ncell_tot, true, c.st, gate);
    end_if(h, c);
    launch_pack(d, h->nblk, h->st, gate);  // every step: the positions changed
    c = begin_if(h, rebuild);
    launch_verlet_build(d, h->nblk, h->tune.reach, c.st);
    end_if(h, c);
  } else {
    launch_drift_bin(d, h->nblk, true, h->st);
    if (drift_done) cudaEventRecord(drift_done, h->st);  // positions final
    launch_scan(d, h->ncell_tot, h->R - 1, h->st);
    launch_scatter_sort_pack(d, h->nblk, h->ncell_tot, true, h->st);
  }
  const bool marks = mode == kPairsF32 && h->prec_any && d.phit;
  launch_density(d, h->nblk, mode, h->tune.reach, verlet, marks, h->cap, h->st, h->tune.dlanes);
  launch_force(d, h->nblk, mode, observe, verlet, h->tune, form_mask(h), h->cap, h->st);
  if (h->prec_any) {
    d.prec_count = h->prec_dev;
    launch_precursor(d, h->nblk, marks, h->st);
  }
  launch_bonded_kick(d, h->nblk, true, h->st);
  if (observe) launch_observe_bonds(d, h->obs_buf, h->n_amp_tot, h->amp_rep, h->st);
  {
    IfScope c = begin_if(h, [&](cudaGraphConditionalHandle ch) {
      launch_cond_cm(ch, d.rep_time, h->R, h->st);
    });
    launch_cmdrift(d, h->nblk, h->R, false, c.st);
    end_if(h, c);
  }
  if (h->chem_on)
    launch_chem(d, h->chem_buf, h->reps_h[0].nblk, h->chem_cfg.n_core, h->chem_amp_cap, false,
                h->st);
  if (observe) launch_observe(d, h->obs_buf, h->nblk, h->n_amp_tot, h->amp_rep, h->R, h->st);
  if (h->chem_on) {
    launch_time_advance(d, h->R, h->st, &h->chem->stop_now);
  } else {
    launch_time_advance(d, h->R, h->st);
  }
}

int enqueue_reorder(idpd_handle* h) {
  launch_reorder(h->d, h->o, h->nblk, 4 * h->n_amp_tot, h->st);
  const size_t n = (size_t)h->n_tot;
  DevState& d = h->d;
  DevState& o = h->o;
  double* dd[12] = {d.px, d.py, d.pz, d.vx, d.vy, d.vz, d.ax, d.ay, d.az, d.dsx, d.dsy, d.dsz};
  double* od[12] = {o.px, o.py, o.pz, o.vx, o.vy, o.vz, o.ax, o.ay, o.az, o.dsx, o.dsy, o.dsz};
  for (int k = 0; k < 12; k++)
    CK(cudaMemcpyAsync(dd[k], od[k], sizeof(double) * n, cudaMemcpyDeviceToDevice, h->st));
  uint32_t* du[6] = {d.id, d.prop, d.amp_id, d.unit, d.orig, d.key};
  uint32_t* ou[6] = {o.id, o.prop, o.amp_id, o.unit, o.orig, o.key};
  for (int k = 0; k < 6; k++)
    CK(cudaMemcpyAsync(du[k], ou[k], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, h->st));
  launch_update_loc(h->d, h->nblk, h->st);
  return IDPD_OK;
}

int pull_to_staging(idpd_handle* h) {
  if (!h->on_device) return IDPD_OK;
  for (int r = 0; r < h->R; r++) {
    Staged& s = h->staged[r];
    const int n = h->n[r];
    s.pos.resize(3 * (size_t)n);
    s.vel.resize(3 * (size_t)n);
    s.acc.resize(3 * (size_t)n);
    s.id.resize(n); s.prop.resize(n); s.amp_id.resize(n); s.unit.resize(n);
    int rc = idpd_download_state(h, r, s.pos.data(), s.vel.data(), s.acc.data(), s.id.data(),
                                 s.prop.data(), s.amp_id.data(), s.unit.data());
    if (rc) return rc;
    if (h->chem_on && r == 0 && h->n_amp[0] != s.n_amp) {
      // molecules appended by reactions: MakeGlobalBondedList over the rows
      const int na = h->n_amp[0];
      s.topol.resize(4 * (size_t)na, kNone);
      s.cf_bend.resize(na, (float)h->params[0].cf_b);
      for (int i = 0; i < n; i++)
        if (s.amp_id[i] != kNone && s.amp_id[i] >= (uint32_t)s.n_amp && s.amp_id[i] < (uint32_t)na &&
            s.unit[i] < 4u)
          s.topol[4 * (size_t)s.amp_id[i] + s.unit[i]] = (uint32_t)i;
      s.n_amp = na;
    }
  }
  return IDPD_OK;
}

}  // namespace

// ============================================================== C ABI

extern "C" {

int idpd_derive_params(const idpd_run_param* rp, idpd_params* out) {
  if (!rp || !out) return fail(nullptr, IDPD_ERR_INVALID_ARG, "null pointer");
  // Parameter::CalcInterCoef (parameter.hpp:138-186) with Tempera = 1,
  // all_unit = 4, Reo = 1.4, arc = 0.9 (parameter.hpp:189-205).
  std::memset(out, 0, sizeof(*out));
  const double T = 1.0, reo = 1.4, arc = 0.9;
  const unsigned all_unit = 4u;
  double c[3][3], g[3][3], s[3][3], m[3][3][3];
  c[1][1] = -2.0 * (rp->kappa + 3.0) / rp->rho_co;
  c[0][0] = c[2][2] = rp->vbb;
  c[0][1] = c[1][0] = rp->chi / (rp->rho_co) + 0.5 * (c[0][0] + c[1][1]);
  c[2][1] = c[1][2] = c[0][1];
  c[2][0] = c[0][2] = c[0][0];
  const double m0 = 1.5 * (rp->kappa + 2.0) / (rp->rho_co * rp->rho_co);
  for (auto& a : m)
    for (auto& b : a)
      for (double& v : b) v = m0;
  m[0][0][0] = 0.0;
  m[2][2][2] = 0.0;
  int k = 0;
  for (int i = 0; i < 3; i++)
    for (int j = i; j < 3; j++) s[i][j] = rp->cf_r_upper[k++];
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++) s[j][i] = s[i][j];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) g[i][j] = 0.5 * s[i][j] * s[i][j] / T;
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (s[i][j] < 0.0) {
        g[i][j] = g[j][i] = 2.0 / ((1.0 / g[i][i]) + (1.0 / g[j][j]));
        s[i][j] = s[j][i] = std::sqrt(2.0 * g[i][j] * T);
      }
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) s[i][j] /= std::sqrt(rp->dt);
  const double mol_energy = (reo * reo * reo) / (double)(all_unit * all_unit);
  const double arc5 = arc * arc * arc * arc * arc;
  const double pi = 3.14159265358979323846;
  const double w2 = -45.0 / ((arc5 * (2.0 * arc - 3.0) + (3.0 * arc - 2.0)) * pi);
  const double w3 = 15.0 / pi;
  const double dum = ((reo * reo * reo * 15.0) / (2.0 * pi * (double)all_unit));
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c[i][j] *= mol_energy * w2;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int q = 0; q < 3; q++) m[i][j][q] *= mol_energy * (2.0 / 3.0) * w3 * dum;
  std::memcpy(out->cf_c, c, sizeof(c));
  std::memcpy(out->cf_g, g, sizeof(g));
  std::memcpy(out->cf_r, s, sizeof(s));
  std::memcpy(out->cf_m, m, sizeof(m));
  out->cf_s = rp->cf_s;
  out->cf_b = rp->cf_b;
  out->cf_b_rigid = rp->cf_b_rigid;
  for (int q = 0; q < 3; q++) out->box[q] = rp->box[q];
  out->dt = rp->dt;
  return IDPD_OK;
}

int idpd_create(const idpd_config* cfg, idpd_handle** out) {
  if (!cfg || !out) return fail(nullptr, IDPD_ERR_INVALID_ARG, "null pointer");
  *out = nullptr;
  if (cfg->n_replicas < 1) return fail(nullptr, IDPD_ERR_INVALID_ARG, "n_replicas must be >= 1");
  if ((cfg->flags & IDPD_CFG_FP64_PAIRS) && (cfg->flags & IDPD_CFG_FP64_KEPT))
    return fail(nullptr, IDPD_ERR_INVALID_ARG,
                "IDPD_CFG_FP64_PAIRS and IDPD_CFG_FP64_KEPT exclude each other");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(nullptr, IDPD_ERR_NO_DEVICE, "no CUDA device visible");
  }
  if (cfg->device < 0 || cfg->device >= ndev)
    return fail(nullptr, IDPD_ERR_INVALID_ARG, "device %d out of range", cfg->device);
  idpd_handle* h = new idpd_handle();
  h->device = cfg->device;
  h->flags = cfg->flags;
  h->sort_period = cfg->sort_period > 0 ? cfg->sort_period : 100;
  h->R = cfg->n_replicas;
  h->params.assign(h->R, idpd_params{});
  h->params_set.assign(h->R, 0);
  h->prec.assign(h->R, idpd_precursor{});
  h->staged.assign(h->R, Staged{});
  h->n.assign(h->R, 0);
  h->n_amp.assign(h->R, 0);
  if (cudaSetDevice(h->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return fail(nullptr, IDPD_ERR_CUDA, "stream / event creation failed");
  }
  *out = h;
  return IDPD_OK;
}

int idpd_destroy(idpd_handle* h) {
  if (!h) return IDPD_OK;
  cudaSetDevice(h->device);
  if (h->dump_thread.joinable()) h->dump_thread.join();
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->dump_dev) cudaFree(h->dump_dev);
  if (h->dump_host) cudaFreeHost(h->dump_host);
  if (h->dump_ready) cudaEventDestroy(h->dump_ready);
  if (h->dump_done) cudaEventDestroy(h->dump_done);
  if (h->dump_st) cudaStreamDestroy(h->dump_st);
  if (h->xst) cudaStreamDestroy(h->xst);
  if (h->cst) cudaStreamDestroy(h->cst);
  if (h->x_drift) cudaEventDestroy(h->x_drift);
  if (h->x_done) cudaEventDestroy(h->x_done);
  if (h->x_mid) cudaEventDestroy(h->x_mid);
  free_all(h);
  if (h->chem) cudaFree(h->chem);
  if (h->walks) walk_destroy(h->walks);
  if (h->obs_rec) cudaFree(h->obs_rec);
  if (h->obs_count) cudaFree(h->obs_count);
  if (h->prec_dev) cudaFree(h->prec_dev);
  if (h->chem_flag_host) cudaFreeHost(h->chem_flag_host);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return IDPD_OK;
}

int idpd_last_error(const idpd_handle* h, char* buf, size_t len) {
  if (!buf || len == 0) return IDPD_ERR_INVALID_ARG;
  const std::string& s = h ? h->err : g_lib_err;
  std::snprintf(buf, len, "%s", s.c_str());
  return IDPD_OK;
}

int idpd_set_params(idpd_handle* h, int32_t r, const idpd_params* p) {
  if (!h || !p) return fail(h, IDPD_ERR_INVALID_ARG, "null pointer");
  if (r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "replica %d out of range", r);
  int rc = check_params(h, p);
  if (rc) return rc;
  const bool geom_changed = !h->params_set[r] ||
                            std::memcmp(h->params[r].box, p->box, sizeof(p->box)) != 0;
  h->params[r] = *p;
  h->params_set[r] = 1;
  if (geom_changed && h->on_device) {
    if ((rc = pull_to_staging(h))) return rc;
    h->layout_dirty = true;
  }
  h->reps_dirty = true;
  if (h->on_device && !h->layout_dirty) {
    // time is device-resident: update it directly
    cudaSetDevice(h->device);
    CK(cudaMemcpyAsync(h->d.rep_time + r, &p->time, sizeof(uint32_t), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return IDPD_OK;
}

int idpd_get_params(const idpd_handle* h, int32_t r, idpd_params* p) {
  if (!h || !p || r < 0 || r >= h->R) return IDPD_ERR_INVALID_ARG;
  *p = h->params[r];
  if (h->on_device) {
    uint32_t t = 0;
    cudaSetDevice(h->device);
    if (cudaMemcpy(&t, h->d.rep_time + r, sizeof(uint32_t), cudaMemcpyDeviceToHost) == cudaSuccess)
      p->time = t;
  }
  return IDPD_OK;
}

int idpd_upload_state(idpd_handle* h, int32_t r, int32_t n, const double* pos, const double* vel,
                      const double* acc, const uint32_t* id, const uint32_t* prop,
                      const uint32_t* amp_id, const uint32_t* unit) {
  if (!h) return fail(nullptr, IDPD_ERR_INVALID_ARG, "null handle");
  if (r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "replica %d out of range", r);
  if (n < 0 || (n > 0 && (!pos || !vel || !id || !prop)))
    return fail(h, IDPD_ERR_INVALID_ARG, "bad size or null array");
  if (!h->params_set[r]) return fail(h, IDPD_ERR_STATE, "set the parameters of replica %d first", r);
  const idpd_params& p = h->params[r];
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) {
      const double x = pos[3 * (size_t)i + k];
      if (!std::isfinite(x) || !std::isfinite(vel[3 * (size_t)i + k]) ||
          (acc && !std::isfinite(acc[3 * (size_t)i + k])))
        return fail(h, IDPD_ERR_NONFINITE, "non-finite value in row %d", i);
      // CheckParticleConfigIsValid (parameter.hpp:456-462)
      if (!(x >= 0.0 && x <= p.box[k]))
        return fail(h, IDPD_ERR_INVALID_ARG, "row %d lies outside the box", i);
    }
    if (prop[i] >= IDPD_PROP_NUM) return fail(h, IDPD_ERR_INVALID_ARG, "row %d: prop %u", i, prop[i]);
  }
  if (h->on_device && !h->layout_dirty) {
    // the device holds the newest state of every replica: bring it back
    // before the layout is rebuilt from the staging buffers
    int rc = pull_to_staging(h);
    if (rc) return rc;
  }
  Staged& s = h->staged[r];
  s.pos.assign(pos, pos + 3 * (size_t)n);
  s.vel.assign(vel, vel + 3 * (size_t)n);
  if (acc)
    s.acc.assign(acc, acc + 3 * (size_t)n);
  else
    s.acc.assign(3 * (size_t)n, 0.0);
  s.id.assign(id, id + n);
  s.prop.assign(prop, prop + n);
  if (amp_id) s.amp_id.assign(amp_id, amp_id + n); else s.amp_id.assign(n, kNone);
  if (unit) s.unit.assign(unit, unit + n); else s.unit.assign(n, kNone);
  s.topol.clear();
  s.cf_bend.clear();
  s.n_amp = 0;
  h->n[r] = n;
  h->n_amp[r] = 0;
  h->layout_dirty = true;
  return IDPD_OK;
}

int idpd_set_dynamics(idpd_handle* h, int32_t r, const double* pos, const double* vel,
                      const double* acc) {
  if (!h || r < 0 || r >= h->R || !pos || !vel || !acc)
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->on_device || h->layout_dirty) {
    // not on the device yet: the rows wait in the staging buffers (caller
    // buffers in device memory are copied over first, never read by the host)
    Staged& s = h->staged[r];
    const size_t n = (size_t)h->n[r];
    if (s.pos.size() != 3 * n) return fail(h, IDPD_ERR_STATE, "upload the state first");
    std::vector<double> tmp[3];
    const double** src[3] = {&pos, &vel, &acc};
    for (int k = 0; k < 3; k++)
      if (device_view(*src[k])) {
        tmp[k].resize(3 * n);
        CK(cudaMemcpy(tmp[k].data(), *src[k], sizeof(double) * 3 * n, cudaMemcpyDefault));
        *src[k] = tmp[k].data();
      }
    const idpd_params& p = h->params[r];
    for (size_t i = 0; i < 3 * n; i++)
      if (!std::isfinite(pos[i]) || !std::isfinite(vel[i]) || !std::isfinite(acc[i]) ||
          !(pos[i] >= 0.0 && pos[i] <= p.box[i % 3]))
        return fail(h, IDPD_ERR_INVALID_ARG, "row %zu: position outside the box or non-finite value", i / 3);
    s.pos.assign(pos, pos + 3 * n);
    s.vel.assign(vel, vel + 3 * n);
    s.acc.assign(acc, acc + 3 * n);
    return IDPD_OK;
  }
  cudaSetDevice(h->device);
  const RepDev& R = h->reps_h[r];
  const size_t n = (size_t)R.n;
  if (n == 0) return IDPD_OK;
  // device buffers are read by the kernel where they lie; host ones are
  // copied to the staging buffer first
  const double* src[3] = {pos, vel, acc};
  const double* dev[3];
  for (int k = 0; k < 3; k++) {
    dev[k] = static_cast<const double*>(device_view(src[k]));
    if (!dev[k]) {
      double* stage = h->xfer + 3 * n * k;
      CK(cudaMemcpyAsync(stage, src[k], 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->st));
      dev[k] = stage;
    }
  }
  // with built kept lists the position change counts as displacement (the
  // next step rebuilds when it is too large); else the lists are rebuilt
  const bool kept = h->d.vdev && !h->vl_dirty && h->tune.skin > 0.0f;
  launch_set_dynamics(h->d, dev[0], dev[1], dev[2], R.row_off, R.n, R.box[0], R.box[1], R.box[2],
                      kept, h->st);
  h->density_valid = false;
  return IDPD_OK;
}

int idpd_num_particles(const idpd_handle* h, int32_t r, int32_t* n) {
  if (!h || !n || r < 0 || r >= h->R) return IDPD_ERR_INVALID_ARG;
  *n = h->n[r];
  return IDPD_OK;
}

int idpd_build_topology(idpd_handle* h, int32_t r, int32_t n_amp, int32_t n_core,
                        const uint32_t* core_amp_id) {
  if (!h || r < 0 || r >= h->R || n_amp < 0 || n_core < 0 || (n_core > 0 && !core_amp_id))
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (h->on_device && !h->layout_dirty) {
    int rc = pull_to_staging(h);
    if (rc) return rc;
  }
  Staged& s = h->staged[r];
  const int n = h->n[r];
  if ((int)s.amp_id.size() != n) return fail(h, IDPD_ERR_STATE, "upload the state first");
  // MakeGlobalBondedList (bdf_calculator.hpp:61-88)
  s.topol.assign(4 * (size_t)n_amp, kNone);
  long long cnt = 0;
  for (int i = 0; i < n; i++) {
    const uint32_t a = s.amp_id[i], u = s.unit[i];
    if (a != kNone && u != kNone) {
      if (a >= (uint32_t)n_amp || u >= 4u)
        return fail(h, IDPD_ERR_INVALID_ARG, "row %d: amp_id %u / unit %u out of range", i, a, u);
      if (s.topol[4 * (size_t)a + u] != kNone)
        return fail(h, IDPD_ERR_INVALID_ARG, "molecule %u unit %u appears twice", a, u);
      s.topol[4 * (size_t)a + u] = (uint32_t)i;
      cnt++;
    } else if (s.prop[i] != IDPD_SOLVENT) {
      return fail(h, IDPD_ERR_INVALID_ARG, "row %d has no molecule but is not solvent", i);
    }
  }
  if (cnt != 4ll * n_amp) return fail(h, IDPD_ERR_INVALID_ARG, "topology incomplete: %lld of %d rows", cnt, 4 * n_amp);
  s.cf_bend.assign(n_amp, (float)h->params[r].cf_b);
  for (int k = 0; k < n_core; k++)
    if (core_amp_id[k] < (uint32_t)n_amp) s.cf_bend[core_amp_id[k]] = (float)h->params[r].cf_b_rigid;
  s.n_amp = n_amp;
  h->n_amp[r] = n_amp;
  h->layout_dirty = true;
  return IDPD_OK;
}

int ensure_xst(idpd_handle* h) {
  if (h->xst) return IDPD_OK;
  CK(cudaStreamCreateWithFlags(&h->xst, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&h->x_drift, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->x_done, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&h->x_mid, cudaEventDisableTiming));
  return IDPD_OK;
}

// A storage-order triple (x, y, z arrays) of one replica and where its rows
// go in upload order (device, managed or host memory; null to skip).
struct RowTriple {
  const double *x, *y, *z;
  double* out;
  int slot;  // staging slot in h->xfer (3 n doubles each)
};

// Gathers the triples into upload order on the step's stream and copies the
// host ones back on the exchange stream, so that each gather after the first
// runs under the previous copy; the step's stream then waits for the copies.
int gather_rows_out(idpd_handle* h, const RepDev& R, const RowTriple* f, int nf) {
  const size_t n = (size_t)R.n;
  bool copied = false;
  for (int k = 0; k < nf; k++) {
    if (!f[k].out) continue;
    double* view = static_cast<double*>(const_cast<void*>(device_view(f[k].out)));
    double* tmp = view ? view : h->xfer + 3 * n * f[k].slot;
    launch_soa_to_aos(f[k].x, f[k].y, f[k].z, h->d.loc, R.row_off, tmp, (int)n, h->st);
    if (view) continue;
    CK(cudaEventRecord(h->x_mid, h->st));
    CK(cudaStreamWaitEvent(h->xst, h->x_mid, 0));
    CK(cudaMemcpyAsync(f[k].out, tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->xst));
    copied = true;
  }
  if (copied) {
    CK(cudaEventRecord(h->x_done, h->xst));
    CK(cudaStreamWaitEvent(h->st, h->x_done, 0));
  }
  return IDPD_OK;
}

int idpd_download_state(idpd_handle* h, int32_t r, double* pos, double* vel, double* acc,
                        uint32_t* id, uint32_t* prop, uint32_t* amp_id, uint32_t* unit) {
  if (!h || r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->on_device || h->layout_dirty) {
    // the staged rows; caller buffers in device memory are written by copies
    const Staged& s = h->staged[r];
    const size_t n = (size_t)h->n[r];
    struct Out { void* dst; const void* src; size_t bytes; } outs[7] = {
        {pos, s.pos.data(), sizeof(double) * 3 * n}, {vel, s.vel.data(), sizeof(double) * 3 * n},
        {acc, s.acc.data(), sizeof(double) * 3 * n}, {id, s.id.data(), sizeof(uint32_t) * n},
        {prop, s.prop.data(), sizeof(uint32_t) * n}, {amp_id, s.amp_id.data(), sizeof(uint32_t) * n},
        {unit, s.unit.data(), sizeof(uint32_t) * n}};
    for (const Out& o : outs) {
      if (!o.dst || o.bytes == 0) continue;
      if (device_view(o.dst))
        CK(cudaMemcpy(o.dst, o.src, o.bytes, cudaMemcpyDefault));
      else
        std::memcpy(o.dst, o.src, o.bytes);
    }
    return IDPD_OK;
  }
  cudaSetDevice(h->device);
  const RepDev& R = h->reps_h[r];
  const int n = R.n;
  if (n == 0) return IDPD_OK;
  const DevState& d = h->d;
  // device buffers are written by the gather directly; host ones through the
  // staging buffer and one copy each
  const RowTriple f3[3] = {{d.px, d.py, d.pz, pos, 0}, {d.vx, d.vy, d.vz, vel, 1},
                           {d.ax, d.ay, d.az, acc, 2}};
  int rc = ensure_xst(h);
  if (!rc) rc = gather_rows_out(h, R, f3, 3);
  if (rc) return rc;
  const uint32_t* uf[4] = {d.id, d.prop, d.amp_id, d.unit};
  uint32_t* uo[4] = {id, prop, amp_id, unit};
  std::vector<uint32_t> orig(n), tmpu(n);
  bool need_u = id || prop || amp_id || unit;
  if (need_u) {
    CK(cudaMemcpyAsync(orig.data(), d.orig + R.row_off, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  for (int k = 0; k < 4; k++) {
    if (!uo[k]) continue;
    CK(cudaMemcpyAsync(tmpu.data(), uf[k] + R.row_off, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (int q = 0; q < n; q++) uo[k][orig[q] - (uint32_t)R.row_off] = tmpu[q];
  }
  CK(cudaStreamSynchronize(h->st));
  return rc;
}

int idpd_download_aux(idpd_handle* h, int32_t r, double* density, double* press, double* nei_cm,
                      double* delta_sumr) {
  if (!h || r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->on_device || h->layout_dirty) return fail(h, IDPD_ERR_STATE, "no device state");
  cudaSetDevice(h->device);
  const RepDev& R = h->reps_h[r];
  const int n = R.n;
  if (n == 0) return IDPD_OK;
  std::vector<uint32_t> orig(n), perm(n);
  CK(cudaMemcpyAsync(orig.data(), h->d.orig + R.row_off, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  auto scatter3 = [&](const std::vector<double>& src, double* out, int w) {
    for (int q = 0; q < n; q++)
      for (int k = 0; k < w; k++)
        out[(size_t)w * (orig[q] - (uint32_t)R.row_off) + k] = src[(size_t)w * q + k];
  };
  if (density && h->density_valid && h->d.dens64 && pair_mode(h) != kPairsF32) {
    // the FP64 arms: their FP64 densities (sorted order), unrounded
    std::vector<double> ds(3 * (size_t)n);
    CK(cudaMemcpyAsync(perm.data(), h->d.perm + R.row_off, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(ds.data(), h->d.dens64 + 3 * (size_t)R.row_off, sizeof(double) * 3 * n,
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    std::vector<double> byrow(3 * (size_t)n);
    for (int sidx = 0; sidx < n; sidx++) {
      const int row = (int)perm[sidx] - R.row_off;
      for (int k = 0; k < 3; k++) byrow[3 * (size_t)row + k] = ds[3 * (size_t)sidx + k];
    }
    scatter3(byrow, density, 3);
  } else if (density) {
    if (!h->density_valid || !h->d.dqx) return fail(h, IDPD_ERR_STATE, "run idpd_density first");
    std::vector<long long> q[3];
    const long long* src[3] = {h->d.dqx, h->d.dqy, h->d.dqz};
    CK(cudaMemcpyAsync(perm.data(), h->d.perm + R.row_off, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->st));
    for (int k = 0; k < 3; k++) {
      q[k].resize(n);
      CK(cudaMemcpyAsync(q[k].data(), src[k] + R.row_off, sizeof(long long) * n, cudaMemcpyDeviceToHost, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    std::vector<double> byrow(3 * (size_t)n);
    for (int sidx = 0; sidx < n; sidx++) {
      const int row = (int)perm[sidx] - R.row_off;
      for (int k = 0; k < 3; k++) byrow[3 * (size_t)row + k] = (double)q[k][sidx] * R.dens_unscale;
    }
    scatter3(byrow, density, 3);
  }
  if (press) {
    if (!h->press64) return fail(h, IDPD_ERR_STATE, "run idpd_force first");
    std::vector<double> b(3 * (size_t)n);
    CK(cudaMemcpyAsync(b.data(), h->press64 + 3 * (size_t)R.row_off, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    scatter3(b, press, 3);
  }
  if (nei_cm) {
    if (!h->cm64) return fail(h, IDPD_ERR_STATE, "run idpd_density first");
    std::vector<double> b(6 * (size_t)n);
    CK(cudaMemcpyAsync(b.data(), h->cm64 + 6 * (size_t)R.row_off, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    scatter3(b, nei_cm, 6);
  }
  if (delta_sumr) {
    std::vector<double> b(3 * (size_t)n), t(n);
    const double* src[3] = {h->d.dsx, h->d.dsy, h->d.dsz};
    for (int k = 0; k < 3; k++) {
      CK(cudaMemcpyAsync(t.data(), src[k] + R.row_off, sizeof(double) * n, cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
      for (int q = 0; q < n; q++) b[3 * (size_t)q + k] = t[q];
    }
    scatter3(b, delta_sumr, 3);
  }
  return IDPD_OK;
}

// ---- fine-grained passes

int idpd_drift(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  launch_drift_bin(h->d, h->nblk, true, h->st);
  // the arrival slots of this binning are not used: reset the cell counts
  CK(cudaMemsetAsync(h->d.cell_cnt, 0, sizeof(int) * h->ncell_tot, h->st));
  h->density_valid = false;
  h->vl_dirty = true;
  return check_device_error(h);
}

int idpd_density(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  if ((rc = ensure_aux(h))) return rc;
  enqueue_cells(h, false);
  launch_density(h->d, h->nblk, pair_mode(h), h->tune.reach, false, false, h->cap, h->st);
  launch_com(h->d, h->nblk, h->cm64, h->cm_cnt, h->st);
  h->density_valid = true;
  h->pairs_valid = true;
  return check_device_error(h);
}

int idpd_force(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  if (!h->density_valid) return fail(h, IDPD_ERR_STATE, "idpd_force needs idpd_density on the same positions");
  if ((rc = ensure_aux(h))) return rc;
  launch_force(h->d, h->nblk, pair_mode(h), true, false, h->tune, form_mask(h), h->cap, h->st);
  launch_fq_to_acc(h->d, h->nblk, h->press64, h->st);
  return check_device_error(h);
}

int idpd_bonded(idpd_handle* h, double* vir) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  if ((rc = ensure_aux(h))) return rc;
  // chain geometry comes from the packed cell-local copies: rebuild them
  enqueue_cells(h, false);
  launch_bonded_fine(h->d, h->n_amp_tot, h->amp_rep, h->vir_part, h->st);
  if ((rc = check_device_error(h))) return rc;
  if (vir) {
    std::vector<double> vp(3 * (size_t)std::max(h->n_amp_tot, 1));
    if (h->n_amp_tot > 0) {
      CK(cudaMemcpyAsync(vp.data(), h->vir_part, sizeof(double) * 3 * h->n_amp_tot, cudaMemcpyDeviceToHost, h->st));
      CK(cudaStreamSynchronize(h->st));
    }
    for (int r = 0; r < h->R; r++) {
      double v[3] = {0.0, 0.0, 0.0};
      const RepDev& R = h->reps_h[r];
      for (int a = 0; a < R.n_amp; a++)
        for (int k = 0; k < 3; k++) v[k] += vp[3 * (size_t)(R.amp_off + a) + k];
      for (int k = 0; k < 3; k++) vir[3 * r + k] = v[k];
    }
  }
  return IDPD_OK;
}

int idpd_kick(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  launch_kick_only(h->d, h->nblk, h->st);
  return check_device_error(h);
}

int idpd_remove_cmdrift(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  launch_cmdrift(h->d, h->nblk, h->R, true, h->st);
  return check_device_error(h);
}

// The loop graph: a WHILE conditional node whose body is the captured step
// followed by k_loop_tail. Returns false (and leaves no graph) where the
// driver refuses any part of it; the steps then go one launch each.
bool build_loop_graph(idpd_handle* h) {
  cudaGraph_t g = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return false;
  bool ok = false;
  cudaGraphConditionalHandle cond;
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t node;
  if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        enqueue_step(h, false);
        launch_loop_tail(cond, h->loop_left, h->chem_on ? &h->chem->stopped : nullptr, h->st);
        const cudaError_t le = cudaGetLastError();
        const cudaError_t ce = cudaStreamEndCapture(h->st, &body);
        ok = le == cudaSuccess && ce == cudaSuccess &&
             cudaGraphInstantiate(&h->graph_loop, g, 0) == cudaSuccess;
      }
    }
  }
  cudaGraphDestroy(g);
  if (!ok) {
    h->graph_loop = nullptr;
    cudaGetLastError();  // the refusal is not an error of the step
  }
  return ok;
}

int idpd_step(idpd_handle* h, int32_t nsteps) {
  if (!h || nsteps < 0) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  if (h->n_tot == 0 || nsteps == 0) return IDPD_OK;
  h->pairs_valid = true;
  if (h->chem_on && h->chem_stopped)
    return fail(h, IDPD_ERR_STATE, "the reaction reached max_amp_num: the run has ended");
  if ((rc = ensure_verlet_ready(h)) || (rc = ensure_phit(h))) return rc;
  std::vector<uint32_t> time;  // step counters, to pick the steps that observe
  if (h->obs_period > 0) {
    if ((rc = ensure_obs(h))) return rc;
    time.resize(h->R);
    CK(cudaMemcpyAsync(time.data(), h->d.rep_time, sizeof(uint32_t) * h->R, cudaMemcpyDeviceToHost,
                       h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  for (int variant = 0; variant < (h->obs_period > 0 ? 2 : 1); variant++) {
    cudaGraphExec_t& ge = variant ? h->graph_obs : h->graph;
    if (ge) continue;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    enqueue_step(h, variant == 1);
    const cudaError_t launch_err = cudaGetLastError();  // a launch refused during capture
    const cudaError_t cap_err = cudaStreamEndCapture(h->st, &g);
    if (cap_err != cudaSuccess || launch_err != cudaSuccess)
      return fail(h, IDPD_ERR_CUDA, "step capture: %s (first launch error: %s)",
                  cudaGetErrorString(cap_err), cudaGetErrorString(launch_err));
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, IDPD_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  const bool loop = nsteps > 1 && !(h->flags & IDPD_CFG_PLAIN_GRAPHS) && !h->loop_failed;
  if (loop && !h->graph_loop && !build_loop_graph(h)) h->loop_failed = true;
  const bool use_loop = loop && h->graph_loop;
  // whether the step `ahead` steps from now observes: some replica's step
  // counter is then a multiple of the period
  auto observes = [&](int ahead) {
    for (uint32_t t : time)
      if (((t + (uint32_t)ahead) % (uint32_t)h->obs_period) == 0u) return true;
    return false;
  };
  CK(cudaEventRecord(h->ev0, h->st));
  for (int k = 0; k < nsteps;) {
    // an observing step is one launch of the observation graph; a run of
    // other steps up to the next storage reorder is one launch of the loop
    const bool obs = !time.empty() && observes(0);
    int c = 1;
    if (!obs && use_loop) {
      const int room = std::max(h->sort_period - h->steps_since_sort, 1);
      while (k + c < nsteps && c < room && !(!time.empty() && observes(c))) c++;
    }
    if (c > 1) {
      launch_loop_set(h->loop_left, c, h->st);
      CK(cudaGraphLaunch(h->graph_loop, h->st));
    } else {
      CK(cudaGraphLaunch(obs ? h->graph_obs : h->graph, h->st));
    }
    for (uint32_t& t : time) t += (uint32_t)c;
    k += c;
    h->steps_since_sort += c;
    if (h->steps_since_sort >= h->sort_period) {
      if ((rc = enqueue_reorder(h))) return rc;
      h->steps_since_sort = 0;
    }
    if (h->chem_on) {  // the reference's loop ends after the step whose event stopped it
      CK(cudaMemcpyAsync(h->chem_flag_host, &h->chem->stopped, sizeof(int), cudaMemcpyDeviceToHost,
                         h->st));
      CK(cudaStreamSynchronize(h->st));
      if (*h->chem_flag_host) {
        h->chem_stopped = true;
        break;
      }
    }
  }
  CK(cudaEventRecord(h->ev1, h->st));
  CK(cudaEventSynchronize(h->ev1));
  CK(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->density_valid = false;
  if ((rc = sync_counts(h))) return rc;
  return check_device_error(h);
}

// One step on host arrays: the rows in as idpd_set_dynamics, one step as
// idpd_step(1) (the same kernels, enqueued directly so that the end of the
// drift can be marked), the rows out as idpd_download_state. Positions are
// final after the drift, so they are gathered and copied back on a second
// stream while the pair passes run; velocities and accelerations follow the
// step. One synchronisation at the end.
int idpd_step_host(idpd_handle* h, int32_t r, double* pos, double* vel, double* acc) {
  if (!h || r < 0 || r >= h->R || !pos || !vel || !acc)
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  cudaSetDevice(h->device);
  if (h->chem_on)
    return fail(h, IDPD_ERR_STATE,
                "the reaction can add particles during the step: use idpd_set_dynamics, "
                "idpd_step and idpd_download_state");
  int rc = idpd_set_dynamics(h, r, pos, vel, acc);
  if (rc) return rc;
  if (!h->on_device || h->layout_dirty) {  // the first step of a new layout
    if ((rc = idpd_step(h, 1))) return rc;
    return idpd_download_state(h, r, pos, vel, acc, nullptr, nullptr, nullptr, nullptr);
  }
  if (h->n_tot == 0) return IDPD_OK;
  h->pairs_valid = true;
  if ((rc = ensure_verlet_ready(h)) || (rc = ensure_phit(h))) return rc;
  bool observe = false;
  if (h->obs_period > 0) {
    if ((rc = ensure_obs(h))) return rc;
    std::vector<uint32_t> time(h->R);
    CK(cudaMemcpyAsync(time.data(), h->d.rep_time, sizeof(uint32_t) * h->R, cudaMemcpyDeviceToHost,
                       h->st));
    CK(cudaStreamSynchronize(h->st));
    for (uint32_t t : time) observe = observe || (t % (uint32_t)h->obs_period) == 0u;
  }
  if ((rc = ensure_xst(h))) return rc;
  const RepDev& R = h->reps_h[r];
  const size_t n = (size_t)R.n;
  const DevState& d = h->d;
  CK(cudaEventRecord(h->ev0, h->st));
  enqueue_step(h, observe, h->x_drift);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return fail(h, IDPD_ERR_CUDA, "step launch: %s", cudaGetErrorString(le));
  CK(cudaEventRecord(h->ev1, h->st));
  // positions: gathered to upload order and copied back during the pair passes
  CK(cudaStreamWaitEvent(h->xst, h->x_drift, 0));
  {
    double* view = static_cast<double*>(const_cast<void*>(device_view(pos)));
    double* tmp = view ? view : h->xfer;
    launch_soa_to_aos(d.px, d.py, d.pz, d.loc, R.row_off, tmp, (int)n, h->xst);
    if (!view) CK(cudaMemcpyAsync(pos, tmp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->xst));
  }
  // velocities and accelerations after the kick, the second gather under the
  // first copy; the step's stream then waits for every copy (a reorder
  // permutes the storage rows: not while they are read)
  const RowTriple f2[2] = {{d.vx, d.vy, d.vz, vel, 1}, {d.ax, d.ay, d.az, acc, 2}};
  if ((rc = gather_rows_out(h, R, f2, 2))) return rc;
  CK(cudaEventRecord(h->x_done, h->xst));
  CK(cudaStreamWaitEvent(h->st, h->x_done, 0));
  if (++h->steps_since_sort >= h->sort_period) {
    if ((rc = enqueue_reorder(h))) return rc;
    h->steps_since_sort = 0;
  }
  CK(cudaStreamSynchronize(h->st));
  CK(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
  h->density_valid = false;
  return check_device_error(h);
}

int idpd_sync(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  CK(cudaStreamSynchronize(h->st));
  return check_device_error(h);
}

int idpd_set_tuning(idpd_handle* h, const idpd_tuning* t) {
  if (!h || !t) return fail(h, IDPD_ERR_INVALID_ARG, "null pointer");
  if (t->reach < 1 || t->reach > 2) return fail(h, IDPD_ERR_INVALID_ARG, "reach must be 1 or 2");
  if (t->reach != 1 && (h->flags & IDPD_CFG_FP64_KEPT))
    return fail(h, IDPD_ERR_INVALID_ARG, "the FP64 engine-algorithm arm runs at reach 1");
  if (t->pair_lanes != 0 && t->pair_lanes != 4 && t->pair_lanes != 8 && t->pair_lanes != 16 &&
      t->pair_lanes != 32)
    return fail(h, IDPD_ERR_INVALID_ARG, "pair_lanes must be 4, 8, 16 or 32 (0: 16)");
  if (t->pair_blocks != 0 && t->pair_blocks != 1 && t->pair_blocks != 2 && t->pair_blocks != 4)
    return fail(h, IDPD_ERR_INVALID_ARG, "pair_blocks must be 1, 2 or 4 (0: 1)");
  if (t->density_lanes != 0 && t->density_lanes != 4 && t->density_lanes != 8 &&
      t->density_lanes != 16 && t->density_lanes != 32)
    return fail(h, IDPD_ERR_INVALID_ARG, "density_lanes must be 4, 8, 16 or 32 (0: 32)");
  if (!(t->skin >= 0.0f && t->skin < 1.0f))
    return fail(h, IDPD_ERR_INVALID_ARG, "skin must be in [0, 1)");
  for (int r = 0; r < h->R; r++)
    for (int k = 0; k < 3 && t->skin > 0.0f; k++)
      if (h->params_set[r] && h->params[r].box[k] < 3.0 * (1.0 + t->skin))
        return fail(h, IDPD_ERR_INVALID_ARG,
                    "skin %g needs every box side >= %g (three cells of the cutoff plus skin)",
                    (double)t->skin, 3.0 * (1.0 + t->skin));
  cudaSetDevice(h->device);
  const bool changed = t->reach != h->tune.reach || t->skin != h->tune.skin;
  const int lanes = t->pair_lanes ? t->pair_lanes : 16, fblk = t->pair_blocks ? t->pair_blocks : 1;
  const int dlanes = t->density_lanes ? t->density_lanes : 32;
  if (lanes != h->tune.lanes || fblk != h->tune.fblk || dlanes != h->tune.dlanes)
    invalidate_graph(h);
  h->tune.dlanes = dlanes;
  h->tune.lanes = lanes;
  h->tune.fblk = fblk;
  h->tune.reach = t->reach;
  h->tune.skin = t->skin;
  if (changed && h->on_device && !h->layout_dirty) {
    int rc = retune_cells(h);
    if (rc) return rc;
    h->vl_dirty = true;
    return ensure_verlet(h);
  }
  return IDPD_OK;
}

int idpd_get_tuning(const idpd_handle* h, idpd_tuning* t) {
  if (!h || !t) return IDPD_ERR_INVALID_ARG;
  std::memset(t, 0, sizeof(*t));
  t->reach = h->tune.reach;
  t->skin = h->tune.skin;
  t->pair_lanes = h->tune.lanes;
  t->pair_blocks = h->tune.fblk;
  t->density_lanes = h->tune.dlanes;
  return IDPD_OK;
}

int idpd_list_rebuilds(idpd_handle* h, uint64_t* rebuilds) {
  if (!h || !rebuilds) return IDPD_ERR_INVALID_ARG;
  *rebuilds = 0;
  if (!h->d.vdev) return IDPD_OK;
  cudaSetDevice(h->device);
  unsigned int n = 0;
  CK(cudaMemcpyAsync(&n, &h->d.vdev->rebuilds, sizeof(n), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  *rebuilds = n;
  return check_device_error(h);
}

int idpd_dump_xyz_async(idpd_handle* h, int32_t replica, const char* path, int32_t append) {
  if (!h || !path || replica < 0 || replica >= h->R)
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  // one frame in flight: the previous one is on disk before its buffers are reused
  if (h->dump_thread.joinable()) h->dump_thread.join();
  const RepDev& R = h->reps_h[replica];
  const int n = R.n;
  const size_t bytes = 16 + (size_t)n * (9 * sizeof(double) + 4 * sizeof(uint32_t));
  if (!h->dump_st) {
    CK(cudaStreamCreateWithFlags(&h->dump_st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&h->dump_ready, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&h->dump_done, cudaEventDisableTiming));
  }
  if (bytes > h->dump_cap) {
    if (h->dump_dev) cudaFree(h->dump_dev);
    if (h->dump_host) cudaFreeHost(h->dump_host);
    h->dump_dev = nullptr;
    h->dump_host = nullptr;
    h->dump_cap = 0;
    if (cudaMalloc(&h->dump_dev, bytes) != cudaSuccess ||
        cudaMallocHost(&h->dump_host, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, IDPD_ERR_CAPACITY, "trajectory frame buffers (%zu bytes)", bytes);
    }
    h->dump_cap = bytes;
  }
  // staging layout: time (u32, padded to 16 bytes), pos, vel, acc (n x 3 doubles
  // each), id, prop, amp_id, unit (n u32 each), all in upload order
  const DevState& d = h->d;
  double* f64 = reinterpret_cast<double*>(h->dump_dev + 16);
  uint32_t* u32 = reinterpret_cast<uint32_t*>(h->dump_dev + 16 + 9 * sizeof(double) * (size_t)n);
  CK(cudaMemcpyAsync(h->dump_dev, d.rep_time + replica, sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                     h->st));
  launch_soa_to_aos(d.px, d.py, d.pz, d.loc, R.row_off, f64, n, h->st);
  launch_soa_to_aos(d.vx, d.vy, d.vz, d.loc, R.row_off, f64 + 3 * (size_t)n, n, h->st);
  launch_soa_to_aos(d.ax, d.ay, d.az, d.loc, R.row_off, f64 + 6 * (size_t)n, n, h->st);
  launch_gather_u32x4(d.id, d.prop, d.amp_id, d.unit, d.loc, R.row_off, u32, n, h->st);
  CK(cudaGetLastError());
  CK(cudaEventRecord(h->dump_ready, h->st));
  CK(cudaStreamWaitEvent(h->dump_st, h->dump_ready, 0));
  CK(cudaMemcpyAsync(h->dump_host, h->dump_dev, bytes, cudaMemcpyDeviceToHost, h->dump_st));
  CK(cudaEventRecord(h->dump_done, h->dump_st));
  const std::string file(path);
  const int dev = h->device;
  h->dump_thread = std::thread([h, file, append, n, dev]() {
    cudaSetDevice(dev);
    int frc = IDPD_OK;
    std::string msg;
    if (cudaEventSynchronize(h->dump_done) != cudaSuccess) {
      frc = IDPD_ERR_CUDA;
      msg = std::string("trajectory frame copy: ") + cudaGetErrorString(cudaGetLastError());
    } else {
      const unsigned char* b = h->dump_host;
      uint32_t t;
      std::memcpy(&t, b, sizeof(t));
      const double* f = reinterpret_cast<const double*>(b + 16);
      const uint32_t* u = reinterpret_cast<const uint32_t*>(b + 16 + 9 * sizeof(double) * (size_t)n);
      frc = idpd_write_xyz(file.c_str(), append, t, n, f, f + 3 * (size_t)n, nullptr,
                           f + 6 * (size_t)n, u, u + n, u + 2 * (size_t)n, u + 3 * (size_t)n);
      if (frc != IDPD_OK) {
        char m[512];
        idpd_last_error(nullptr, m, sizeof(m));
        msg = m;
      }
    }
    if (frc != IDPD_OK && h->dump_rc == IDPD_OK) {
      h->dump_rc = frc;
      h->dump_msg = msg;
    }
  });
  return IDPD_OK;
}

int idpd_dump_wait(idpd_handle* h) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  if (h->dump_thread.joinable()) h->dump_thread.join();
  const int rc = h->dump_rc;
  h->dump_rc = IDPD_OK;
  if (rc != IDPD_OK) return fail(h, rc, "trajectory frame: %s", h->dump_msg.c_str());
  return IDPD_OK;
}

int idpd_pair_count(idpd_handle* h, int32_t replica, uint64_t* ordered_pairs) {
  if (!h || !ordered_pairs) return fail(h, IDPD_ERR_INVALID_ARG, "null pointer");
  if (replica < 0 || replica >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "replica %d out of range", replica);
  *ordered_pairs = 0;
  if (!h->on_device || !h->pairs_valid) return IDPD_OK;
  cudaSetDevice(h->device);
  const RepDev& R = h->reps_h[replica];
  unsigned long long sum = 0;
  launch_sum_pairs(h->d.npair, R.row_off, R.n, h->pair_sum, h->st);
  CK(cudaMemcpyAsync(&sum, h->pair_sum, sizeof(sum), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  *ordered_pairs = sum;
  return check_device_error(h);
}

int idpd_last_step_ms(const idpd_handle* h, float* ms) {
  if (!h || !ms) return IDPD_ERR_INVALID_ARG;
  *ms = h->last_ms;
  return IDPD_OK;
}

int idpd_profile_step(idpd_handle* h, char* names, size_t names_len, float* ms, int32_t max_k,
                      int32_t* n_k) {
  if (!h || !names || !ms || !n_k) return fail(h, IDPD_ERR_INVALID_ARG, "null pointer");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  const int mode = pair_mode(h);
  std::vector<cudaEvent_t> ev(10);
  for (auto& e : ev) CK(cudaEventCreate(&e));
  const char* nm[9] = {"drift_bin", "scan", "scatter_sort_pack", "list_build", "density",
                       "force", "bonded_kick", "cmdrift", "time"};
  int rc2 = ensure_verlet_ready(h);
  if (rc2) return rc2;
  DevState d = h->d;
  d.dqx = d.dqy = d.dqz = nullptr;
  const bool verlet = d.vdev && h->tune.skin > 0.0f && mode != kPairsF64;
  const int* gate = verlet ? &d.vdev->rebuild : nullptr;
  CK(cudaEventRecord(ev[0], h->st));
  if (verlet) {
    launch_drift_disp(d, h->nblk, h->st);
    launch_vl_decide(d, h->st);
    launch_bin_gated(d, h->nblk, h->st);
  } else {
    launch_drift_bin(d, h->nblk, true, h->st);
  }
  CK(cudaEventRecord(ev[1], h->st));
  launch_scan(d, h->ncell_tot, h->R - 1, h->st, gate);
  CK(cudaEventRecord(ev[2], h->st));
  launch_scatter_sort_pack(d, h->nblk, h->ncell_tot, true, h->st, gate);
  CK(cudaEventRecord(ev[3], h->st));
  if (verlet) launch_verlet_build(d, h->nblk, h->tune.reach, h->st);
  CK(cudaEventRecord(ev[4], h->st));
  h->pairs_valid = true;
  launch_density(d, h->nblk, mode, h->tune.reach, verlet, false, h->cap, h->st, h->tune.dlanes);
  CK(cudaEventRecord(ev[5], h->st));
  launch_force(d, h->nblk, mode, false, verlet, h->tune, form_mask(h), h->cap, h->st);
  CK(cudaEventRecord(ev[6], h->st));
  launch_bonded_kick(d, h->nblk, true, h->st);
  CK(cudaEventRecord(ev[7], h->st));
  launch_cmdrift(d, h->nblk, h->R, false, h->st);
  CK(cudaEventRecord(ev[8], h->st));
  launch_time_advance(d, h->R, h->st);
  CK(cudaEventRecord(ev[9], h->st));
  CK(cudaEventSynchronize(ev[9]));
  std::string all;
  int k = 0;
  for (; k < 9 && k < max_k; k++) {
    CK(cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]));
    all += nm[k];
    all += "\n";
  }
  *n_k = k;
  std::snprintf(names, names_len, "%s", all.c_str());
  for (auto& e : ev) cudaEventDestroy(e);
  h->density_valid = false;
  if (++h->steps_since_sort >= h->sort_period) {
    if ((rc = enqueue_reorder(h))) return rc;
    h->steps_since_sort = 0;
  }
  return check_device_error(h);
}

// Saru test draws on the device: the keys in, the draws out. One device
// block holds keys and draws and is freed on every path.
static int saru_draws(int32_t n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                      int32_t draws, uint32_t* out_u, float* out_n) {
  idpd_handle* h = nullptr;
  const size_t nk = (size_t)n, nd = out_u ? nk * (size_t)draws : nk;
  uint32_t* buf = nullptr;
  CK(cudaMalloc((void**)&buf, 4 * (3 * nk + nd)));
  cudaError_t e = cudaSuccess;
  const uint32_t* src[3] = {s1, s2, s3};
  for (int k = 0; k < 3 && e == cudaSuccess; k++)
    e = cudaMemcpy(buf + k * nk, src[k], 4 * nk, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    uint32_t* dout = buf + 3 * nk;
    launch_saru_test(n, buf, buf + nk, buf + 2 * nk, out_u ? draws : 0, out_u ? dout : nullptr,
                     out_u ? nullptr : reinterpret_cast<float*>(dout), 0);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpy(out_u ? (void*)out_u : (void*)out_n, dout, 4 * nd, cudaMemcpyDeviceToHost);
  }
  cudaFree(buf);
  if (e != cudaSuccess) return fail(nullptr, IDPD_ERR_CUDA, "saru draws: %s", cudaGetErrorString(e));
  return IDPD_OK;
}

int idpd_saru_u32(int32_t n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                  int32_t draws, uint32_t* out) {
  if (n < 0 || draws < 0 || (n > 0 && (!s1 || !s2 || !s3 || !out)))
    return fail(nullptr, IDPD_ERR_INVALID_ARG, "bad argument");
  if (n == 0 || draws == 0) return IDPD_OK;
  return saru_draws(n, s1, s2, s3, draws, out, nullptr);
}

int idpd_saru_nrml_f32(int32_t n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                       float* out) {
  if (n < 0 || (n > 0 && (!s1 || !s2 || !s3 || !out)))
    return fail(nullptr, IDPD_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return IDPD_OK;
  return saru_draws(n, s1, s2, s3, 0, nullptr, out);
}

int idpd_cell_order(idpd_handle* h, int32_t r, uint32_t* cell_of_row, uint32_t* perm_out) {
  if (!h || r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  enqueue_cells(h, false);
  const RepDev& R = h->reps_h[r];
  const int n = R.n;
  std::vector<uint32_t> key(n), perm(n), orig(n);
  CK(cudaMemcpyAsync(key.data(), h->d.key + R.row_off, 4 * (size_t)n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(perm.data(), h->d.perm + R.row_off, 4 * (size_t)n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(orig.data(), h->d.orig + R.row_off, 4 * (size_t)n, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int q = 0; q < n; q++) {
    const uint32_t up = orig[q] - (uint32_t)R.row_off;
    if (cell_of_row) cell_of_row[up] = key[q] - (uint32_t)R.cell_off;
    if (perm_out) perm_out[q] = orig[perm[q] - (uint32_t)R.row_off] - (uint32_t)R.row_off;
  }
  h->density_valid = false;
  return check_device_error(h);
}

int idpd_set_observe(idpd_handle* h, int32_t period, int32_t capacity) {
  if (!h || period < 0 || (period > 0 && capacity < 1))
    return fail(h, IDPD_ERR_INVALID_ARG, "period >= 0 and capacity >= 1 required");
  cudaSetDevice(h->device);
  CK(cudaStreamSynchronize(h->st));
  if (period > 0 && capacity != h->obs_cap) {
    if (h->walks) walk_destroy(h->walks);
  if (h->obs_rec) cudaFree(h->obs_rec);
    h->obs_rec = nullptr;
    CK(cudaMalloc((void**)&h->obs_rec, sizeof(idpd_observation) * (size_t)capacity));
    if (!h->obs_count) CK(cudaMalloc((void**)&h->obs_count, sizeof(int)));
    h->obs_cap = capacity;
  }
  if (h->obs_count) CK(cudaMemsetAsync(h->obs_count, 0, sizeof(int), h->st));
  h->obs_period = period;
  invalidate_graph(h);
  return IDPD_OK;
}

int idpd_get_observations(idpd_handle* h, idpd_observation* out, int32_t max, int32_t* n) {
  if (!h || !n || max < 0 || (max > 0 && !out)) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  *n = 0;
  if (!h->obs_count) return IDPD_OK;
  cudaSetDevice(h->device);
  int cnt = 0;
  CK(cudaMemcpyAsync(&cnt, h->obs_count, sizeof(int), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  const int have = std::min(cnt, h->obs_cap);
  std::vector<idpd_observation> rec(have);
  if (have > 0)
    CK(cudaMemcpyAsync(rec.data(), h->obs_rec, sizeof(idpd_observation) * have,
                       cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemsetAsync(h->obs_count, 0, sizeof(int), h->st));
  CK(cudaStreamSynchronize(h->st));
  // replicas finish in any order within a step: order by (time, replica)
  std::stable_sort(rec.begin(), rec.end(), [](const idpd_observation& a, const idpd_observation& b) {
    return a.time != b.time ? a.time < b.time : a.replica < b.replica;
  });
  const int k = std::min(have, max);
  for (int i = 0; i < k; i++) out[i] = rec[i];
  *n = k;
  if (cnt > h->obs_cap || have > max)
    return fail(h, IDPD_ERR_CAPACITY, "%d observations recorded, %d returned", cnt, k);
  return IDPD_OK;
}

int idpd_density_profile(idpd_handle* h, int32_t r, int32_t axis, int32_t nbins, double* out) {
  if (!h || r < 0 || r >= h->R || axis < 0 || axis > 2 || nbins < 1 || !out)
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  const RepDev& R = h->reps_h[r];
  unsigned long long* hist = nullptr;
  CK(cudaMallocAsync((void**)&hist, sizeof(unsigned long long) * 3 * nbins, h->st));
  CK(cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * 3 * nbins, h->st));
  launch_density_profile(h->d, r, R.row_off, R.n, axis, nbins, hist, h->st);
  std::vector<unsigned long long> c(3 * (size_t)nbins);
  CK(cudaMemcpyAsync(c.data(), hist, sizeof(unsigned long long) * 3 * nbins, cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaFreeAsync(hist, h->st));
  CK(cudaStreamSynchronize(h->st));
  const double vol = R.box[0] * R.box[1] * R.box[2] / (double)nbins;
  for (size_t k = 0; k < c.size(); k++) out[k] = (double)c[k] / vol;
  return check_device_error(h);
}

int idpd_rdf(idpd_handle* h, int32_t r, int32_t nbins, double r_max, double* out) {
  if (!h || r < 0 || r >= h->R || nbins < 1 || nbins > 1024 || !out || !(r_max > 0.0 && r_max <= 2.0))
    return fail(h, IDPD_ERR_INVALID_ARG, "nbins in [1, 1024], r_max in (0, 2] required");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  const RepDev& R = h->reps_h[r];
  // search cells have side >= 1 / reach: m layers cover r_max
  const int m = (int)std::ceil(r_max * (double)R.reach - 1e-12);
  for (int k = 0; k < 3; k++)
    if (R.nc[k] < 2 * m + 1)
      return fail(h, IDPD_ERR_INVALID_ARG, "rdf up to %g needs every box side >= %d", r_max,
                  2 * (int)std::ceil(r_max) + 1);
  enqueue_cells(h, false);
  unsigned long long* hist = nullptr;
  CK(cudaMallocAsync((void**)&hist, sizeof(unsigned long long) * nbins, h->st));
  CK(cudaMemsetAsync(hist, 0, sizeof(unsigned long long) * nbins, h->st));
  launch_rdf(h->d, r, R.row_off, R.n, nbins, r_max, m, hist, h->st);
  std::vector<unsigned long long> c(nbins);
  CK(cudaMemcpyAsync(c.data(), hist, sizeof(unsigned long long) * nbins, cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaFreeAsync(hist, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->density_valid = false;
  const double n = (double)R.n, rho = n / (R.box[0] * R.box[1] * R.box[2]);
  const double pi = 3.14159265358979323846, dr = r_max / nbins;
  for (int k = 0; k < nbins; k++) {
    const double r1 = k * dr, r2 = (k + 1) * dr;
    const double shell = 4.0 / 3.0 * pi * (r2 * r2 * r2 - r1 * r1 * r1);
    out[k] = n > 0 ? (double)c[k] / (n * rho * shell) : 0.0;
  }
  return check_device_error(h);
}

int idpd_dispatch_walks(idpd_handle* h, int32_t kind, int32_t tag, int32_t n_walk,
                        const void* const* epi, const int32_t* n_epi, const void* const* epj,
                        const int32_t* n_epj) {
  if (!h || (kind != IDPD_WALK_DENSITY && kind != IDPD_WALK_FORCE) || n_walk < 0 ||
      (n_walk > 0 && (!epi || !n_epi || !epj || !n_epj)))
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->params_set[0]) return fail(h, IDPD_ERR_STATE, "set the parameters of replica 0 first");
  cudaSetDevice(h->device);
  if (!h->walks) h->walks = walk_create();
  idpd_params p = h->params[0];
  if (h->on_device)  // the step counter lives on the device
    CK(cudaMemcpy(&p.time, h->d.rep_time, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  RepDev R{};
  fill_repdev(R, p, 1, 0.0f);
  std::string err;
  const int rc = walk_dispatch(h->walks, h->st, R, p, kind, tag, n_walk, epi, n_epi, epj, n_epj, err);
  if (rc) return fail(h, rc, "dispatch_walks: %s", err.c_str());
  return IDPD_OK;
}

int idpd_retrieve_walks(idpd_handle* h, int32_t kind, int32_t tag, int32_t n_walk,
                        const int32_t* ni, void* const* result) {
  if (!h || (kind != IDPD_WALK_DENSITY && kind != IDPD_WALK_FORCE) || n_walk < 0 ||
      (n_walk > 0 && (!ni || !result)))
    return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->walks) return fail(h, IDPD_ERR_STATE, "no walks dispatched");
  cudaSetDevice(h->device);
  std::string err;
  const int rc = walk_retrieve(h->walks, kind, tag, n_walk, ni, result, err);
  if (rc) return fail(h, rc, "retrieve_walks: %s", err.c_str());
  return IDPD_OK;
}

int idpd_set_precursor(idpd_handle* h, int32_t r, const idpd_precursor* cfg) {
  if (!h) return fail(h, IDPD_ERR_INVALID_ARG, "null handle");
  if (r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "replica %d out of range", r);
  idpd_precursor q{};
  if (cfg && cfg->enabled) {
    if (cfg->prop_from >= IDPD_PROP_NUM || cfg->prop_near >= IDPD_PROP_NUM ||
        cfg->prop_to >= IDPD_PROP_NUM)
      return fail(h, IDPD_ERR_INVALID_ARG, "properties must be below %d", IDPD_PROP_NUM);
    q = *cfg;
    q.enabled = 1;
  }
  cudaSetDevice(h->device);
  if (!h->prec_dev) CK(cudaMalloc((void**)&h->prec_dev, sizeof(unsigned long long) * h->R));
  if (!h->prec_any) CK(cudaMemsetAsync(h->prec_dev, 0, sizeof(unsigned long long) * h->R, h->st));
  CK(cudaMemsetAsync(h->prec_dev + r, 0, sizeof(unsigned long long), h->st));
  h->prec[r] = q;
  h->prec_any = false;
  for (const idpd_precursor& p : h->prec) h->prec_any = h->prec_any || p.enabled;
  h->reps_dirty = true;
  invalidate_graph(h);
  return IDPD_OK;
}

int idpd_precursor_count(idpd_handle* h, int32_t r, uint64_t* conversions) {
  if (!h || !conversions) return fail(h, IDPD_ERR_INVALID_ARG, "null pointer");
  if (r < 0 || r >= h->R) return fail(h, IDPD_ERR_INVALID_ARG, "replica %d out of range", r);
  *conversions = 0;
  if (!h->prec_dev) return IDPD_OK;
  cudaSetDevice(h->device);
  unsigned long long c = 0;
  CK(cudaMemcpyAsync(&c, h->prec_dev + r, sizeof(c), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  *conversions = c;
  return IDPD_OK;
}

int idpd_set_chem(idpd_handle* h, int32_t r, const idpd_chem_config* cfg) {
  if (!h || r != 0) return fail(h, IDPD_ERR_INVALID_ARG, "the reaction acts on replica 0");
  cudaSetDevice(h->device);
  if (!cfg) {
    if (h->chem_on) {
      int rc = pull_to_staging(h);
      if (rc) return rc;
      h->chem_on = false;
      h->chem_stopped = false;
      h->layout_dirty = true;
    }
    return IDPD_OK;
  }
  if (h->R != 1) return fail(h, IDPD_ERR_INVALID_ARG, "the reaction needs a one-replica handle");
  if (!h->params_set[0]) return fail(h, IDPD_ERR_STATE, "set the parameters first");
  if (cfg->n_core < 0 || cfg->n_core > IDPD_CHEM_MAX_CORE || cfg->reserve_amp < 0)
    return fail(h, IDPD_ERR_INVALID_ARG, "n_core must be in [0, %d], reserve_amp >= 0",
                IDPD_CHEM_MAX_CORE);
  const idpd_chem_params& q = cfg->p;
  const double vals[6] = {q.p_thresld, q.eps, q.influ_rad, q.influ_hei, q.influ_dep, q.influ_grd};
  for (double v : vals)
    if (!std::isfinite(v)) return fail(h, IDPD_ERR_INVALID_ARG, "non-finite reaction parameter");
  for (int k = 0; k < 3; k++)
    if (h->params[0].box[k] < 5.0)
      return fail(h, IDPD_ERR_INVALID_ARG, "the core geometry needs every box side >= 5");
  if (h->on_device && !h->layout_dirty) {  // keep the current state through the re-layout
    int rc = sync_counts(h);
    if (rc) return rc;
    if ((rc = pull_to_staging(h))) return rc;
  }
  if (!h->chem) {
    CK(cudaMalloc((void**)&h->chem, sizeof(ChemDev)));
    CK(cudaMallocHost((void**)&h->chem_flag_host, sizeof(int)));
  }
  ChemDev c;
  std::memset(&c, 0, sizeof(c));
  c.mt[0] = cfg->mt_seed;  // init_genrand (Matsumoto & Nishimura, mt19937ar)
  for (int i = 1; i < 624; i++) c.mt[i] = 1812433253u * (c.mt[i - 1] ^ (c.mt[i - 1] >> 30)) + (uint32_t)i;
  c.mti = 624;
  c.p_thresld = q.p_thresld;
  c.eps = q.eps;
  c.influ_rad = q.influ_rad;
  c.influ_hei = q.influ_hei;
  c.influ_dep = q.influ_dep;
  c.influ_grd = q.influ_grd;
  c.amp_num = (uint32_t)h->n_amp[0];
  c.max_amp_num = q.max_amp_num;
  c.beg_chem = cfg->beg_chem;
  c.n_core = cfg->n_core;
  for (int k = 0; k < cfg->n_core; k++) c.core_id[k] = cfg->core_ptcl_id[k];
  c.cf_bend = (float)h->params[0].cf_b;
  CK(cudaMemcpyAsync(h->chem, &c, sizeof(c), cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->chem_cfg = *cfg;
  h->chem_on = true;
  h->chem_stopped = false;
  h->layout_dirty = true;
  invalidate_graph(h);
  return IDPD_OK;
}

int idpd_chem_event(idpd_handle* h, int32_t* cont) {
  if (!h) return IDPD_ERR_INVALID_ARG;
  if (!h->chem_on) return fail(h, IDPD_ERR_STATE, "the reaction is not enabled (idpd_set_chem)");
  if (h->chem_stopped) return fail(h, IDPD_ERR_STATE, "the reaction reached max_amp_num");
  cudaSetDevice(h->device);
  int rc = commit(h);
  if (rc) return rc;
  enqueue_cells(h, false);
  launch_chem(h->d, h->chem_buf, h->reps_h[0].nblk, h->chem_cfg.n_core, h->chem_amp_cap, true,
              h->st);
  CK(cudaMemcpyAsync(h->chem_flag_host, &h->chem->stopped, sizeof(int), cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaStreamSynchronize(h->st));
  h->chem_stopped = *h->chem_flag_host != 0;
  if (cont) *cont = h->chem_stopped ? 0 : 1;
  h->density_valid = false;
  if ((rc = sync_counts(h))) return rc;
  return check_device_error(h);
}

int idpd_chem_get_info(idpd_handle* h, int32_t r, idpd_chem_info* info, uint32_t* targets,
                       int32_t cap) {
  if (!h || r != 0 || !info || cap < 0) return fail(h, IDPD_ERR_INVALID_ARG, "bad argument");
  if (!h->chem_on || !h->chem) return fail(h, IDPD_ERR_STATE, "the reaction is not enabled");
  cudaSetDevice(h->device);
  ChemDev c;
  CK(cudaMemcpyAsync(&c, h->chem, sizeof(c), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  std::memset(info, 0, sizeof(*info));
  info->n_targets = c.n_targets;
  info->events = c.events;
  info->stopped = c.stopped;
  info->amp_num = c.amp_num;
  for (int k = 0; k < IDPD_CHEM_MAX_CORE && k < kChemMaxCore; k++)
    for (int q = 0; q < 9; q++) info->core_raw[k][q] = c.core_raw[k][q];
  info->n_core = c.events > 0 ? c.n_core : 0;
  for (int k = 0; k < info->n_core && k < IDPD_CHEM_MAX_CORE; k++)
    for (int q = 0; q < 3; q++) {
      info->h2t[k][q] = c.core_n[k][q];
      info->core_h[k][q] = c.core_h[k][q];
    }
  const int nt = std::min(c.n_targets, cap);
  if (targets && nt > 0 && h->chem_buf.targets) {
    CK(cudaMemcpyAsync(targets, h->chem_buf.targets, sizeof(uint32_t) * 2 * nt,
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
  }
  return IDPD_OK;
}

}  // extern "C"
