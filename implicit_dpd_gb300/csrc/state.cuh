// Device buffers of one engine handle and the host-side launchers of every
// kernel. The layout in HBM:
//   storage order (one row per particle, replicas packed in replica order):
//     FP64 SoA pos/vel/acc/delta_sumr, u32 id/prop/amp_id/unit, replica, the
//     upload row (orig) used to hand rows back in upload order;
//   sorted order (rows grouped by cell, rebuilt every step):
//     perm (sorted -> storage), rank (storage -> sorted), scell (global cell),
//     float4 posf (cell-local position, prop bits), velf (velocity, id bits),
//     densf (partial densities), int64 fixed-point pair force fq (x, y, z and
//     a pad word per row: the three sums of a row share one 32-byte sector);
//   cells: per-cell count and start (exclusive prefix) over all replicas.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "common.cuh"
#include "idpd_engine.h"

namespace idpd {

struct DevState {
  // ---- storage order
  double *px, *py, *pz;
  double *vx, *vy, *vz;
  double *ax, *ay, *az;
  double *dsx, *dsy, *dsz;  // delta_sumr
  uint32_t *id, *prop, *amp_id, *unit;
  uint32_t* orig;  // upload row of this storage row
  uint32_t* loc;   // storage row of each upload row (inverse of orig)
  // ---- cell build (per step)
  uint32_t* key;   // global cell of storage row
  uint32_t* slot;  // arrival slot inside the cell
  int* cell_cnt;   // [ncell_tot]
  int* cell_start; // [ncell_tot + 1]
  int* scan_part;  // block partial sums of the scan
  // ---- sorted order
  uint32_t* perm;
  uint32_t* rank;
  uint32_t* scell;
  float4 *posf, *velf, *densf;
  float4* poslo;               // low-order parts of the cell-local position
  uint32_t* nbl;               // [N * kNbrCap] in-range neighbours of pass 1 (sorted order)
  uint16_t* nbn;               // [N] list length (owned pairs), or 0xffff when it overflowed
  long long* fq;               // [4N] pair force, 2^-26 fixed point: x, y, z, pad per sorted row
  long long* pq;               // [4N] per-particle virial, same layout (fine-grained API, observation)
  long long *dqx, *dqy, *dqz;  // partial densities in RepDev::dens_unscale units (fine-grained API only)
  double* dens64;              // [3N] partial densities of the FP64 arms (sorted order)
  double* svel;                // [4N] FP64 velocity per sorted row (FP64 engine-algorithm arm)
  unsigned long long* dsum;    // [4N] pass-1 partial densities by property, fixed point (zero between passes)
  // ---- topology
  uint32_t* topol;  // [4 * total molecules] storage rows
  float* cf_bend;   // [total molecules]
  // ---- replicas and launch maps
  RepDev* reps;
  RepTab64* tab64;
  uint32_t* rep_time;  // Parameter::time per replica
  int* blk_rep;
  int* blk_row;
  // ---- reductions
  double* blk_part;  // [n_blocks * 3]
  uint32_t* npair;   // [N] ordered pairs within the cutoff (r < 1, i != j) of each sorted row,
                     // counted by pass 1 (2 x the owned pairs in the once-per-pair passes)
  double* rep_mean;  // [R * 3]
  int* err;          // device error word (0 = ok)
  unsigned long long* prec_count;  // [R] precursor conversions per replica
  uint8_t* phit;                   // [N] pass 1 took a pair of the conversion's properties
  // ---- neighbour lists kept between rebuilds (null when the skin is 0)
  uint32_t* vl;                // [N * kVerletCap] pairs within 1 + skin at the last rebuild
  uint16_t* vn;                // [N] list length, or 0xffff when it did not fit
  float* okey;                 // [N] cell-local x at the last build (pair ownership)
  double *drx, *dry, *drz;     // delta_sumr at the last rebuild (sorted order)
  struct VerletDev* vdev;
};

// The rebuild schedule of the kept lists: a rebuild when any particle moved
// more than half the skin since the last one, or when forced (new layout,
// new positions, particles added).
struct VerletDev {
  int rebuild;          // this step rebuilds the cells and lists
  int force;            // the next step must rebuild
  unsigned int maxd2;   // bits of the largest squared displacement (float, >= 0)
  float thr2;           // (skin / 2)^2 less a margin
  float rv2;            // build cutoff (1 + skin)^2 plus a margin
  unsigned int rebuilds;
};

// Error codes written by kernels into DevState::err.
enum : int { kErrNone = 0, kErrCellOverflow = 1, kErrBadCell = 2, kErrListOverflow = 3,
             kErrNonFinite = 4, kErrComBox = 5, kErrChemCapacity = 6, kErrDensPairs = 7 };
// Pairs within the cutoff of one particle that pass 1 can weigh (its lanes
// keep 32-bit partial densities: (18 + kDensPairsMax / 32) * 2^23 < 2^32).
constexpr int kDensPairsMax = 15000;

// Device state of ChemManager (chemmanager.hpp:3-282) for replica 0 of a
// one-replica handle: the MT19937 generator of PS::MT, the Parameter
// members the event reads, and what the last event did.
constexpr int kChemMaxCore = 8;
struct ChemDev {
  uint32_t mt[624];  // mt19937ar state (raw words) and its read index
  int mti;
  int active;        // an event runs in this step
  int stopped;       // amp_num reached max_amp_num: RandomChemEvent returned false
  int stop_now;      // the event of this step stopped the run (time is not advanced)
  double p_thresld, eps, influ_rad, influ_hei, influ_dep, influ_grd;
  uint32_t amp_num, max_amp_num, beg_chem;
  int n_core;
  uint32_t core_id[kChemMaxCore];
  int core_row[kChemMaxCore];        // storage row of each core particle (-1: absent)
  double core_raw[kChemMaxCore][9];  // GetCorePos: head pos, hydrophobic cm, hydrophilic cm
  double core_h[kChemMaxCore][3];    // projected core position (DetermineTargetIdWithCorePos)
  double core_n[kChemMaxCore][3];    // unit head-to-tail vector
  int n_targets;     // targets of the last event
  int events;        // events run
  int row_cap, amp_cap, target_cap;  // rows, molecules and targets the buffers hold
  float cf_bend;     // bend coefficient of new molecules (cf_b)
};

constexpr int kRowBlock = 128;  // rows per block of row-block launches
constexpr int kNbrCap = 512;    // neighbour-list slots per particle
constexpr int kVerletCap = 512;  // kept-list slots per particle

// kernels_cells.cu
void launch_drift_bin(const DevState& d, int nblk, bool do_drift, cudaStream_t st);
// start[ncell_tot] = reps[last_rep].row_off + reps[last_rep].n, read on the
// device (the particle count can grow on the device).
void launch_scan(const DevState& d, int ncell_tot, int last_rep, cudaStream_t st,
                 const int* gate = nullptr);
// Steps with kept lists: drift plus the largest displacement since the last
// rebuild, the rebuild decision, and the binning of rebuild steps.
void launch_drift_disp(const DevState& d, int nblk, cudaStream_t st);
void launch_vl_decide(const DevState& d, cudaStream_t st);
void launch_bin_gated(const DevState& d, int nblk, cudaStream_t st);
// gate (may be null): device flag; when 0 the sort is skipped and the pack
// keeps each slot's cell of the last rebuild.
void launch_scatter_sort_pack(const DevState& d, int nblk, int ncell_tot, bool stable,
                              cudaStream_t st, const int* gate = nullptr);
// The two halves of launch_scatter_sort_pack: rows to sorted slots and the
// stable order within cells; the FP32 copies of the pair passes.
void launch_scatter_sort(const DevState& d, int nblk, int ncell_tot, bool stable, cudaStream_t st,
                         const int* gate = nullptr);
void launch_pack(const DevState& d, int nblk, cudaStream_t st, const int* gate = nullptr);
// Conditions of the IF nodes of a captured step: the rebuild flag, and
// whether the centre-of-mass drift removal is due for some replica.
void launch_cond_flag(cudaGraphConditionalHandle cond, const int* flag, cudaStream_t st);
void launch_cond_cm(cudaGraphConditionalHandle cond, const uint32_t* rep_time, int R,
                    cudaStream_t st);
void launch_reorder(const DevState& d, const DevState& o, int nblk, int n_topol,
                    cudaStream_t st);
void launch_update_loc(const DevState& d, int nblk, cudaStream_t st);
// Counting-sort pieces on raw arrays: exclusive scan of cnt into start
// (start[ncell] = n_tot, cnt cleared; part holds ncell / 4096 + 1 ints) and
// the per-cell ascending order of perm.
void launch_scan_raw(int* cnt, int* start, int* part, int ncell, int n_tot, cudaStream_t st);
void launch_cell_sort_raw(uint32_t* perm, const int* start, int ncell, cudaStream_t st);
// Binning of n rows (x y z triples) on one grid of nc cells per axis, and the
// scatter of rows to their sorted slots.
void launch_bin_rows(const double* pos, int n, const double inv_cs[3], const int nc[3],
                     uint32_t* cell, uint32_t* slot, int* cnt, cudaStream_t st);
void launch_scatter_rows(const uint32_t* cell, const uint32_t* slot, const int* start, int n,
                         uint32_t* perm, cudaStream_t st);

// engine.cu: sets the message that idpd_last_error returns for a NULL handle.
void set_library_error(const char* msg);

// kernels_pairs.cu
// Arithmetic of the pair passes: the FP32 engine, the plain FP64 kernels
// (IDPD_CFG_FP64_PAIRS) or the engine's algorithm in FP64 (IDPD_CFG_FP64_KEPT).
enum PairMode : int { kPairsF32 = 0, kPairsF64 = 1, kPairsF64Kept = 2 };
struct PairTuning {
  int reach;       // 1: cells of the cutoff, 27-cell stencil; 2: half cells, 125-cell stencil
  float skin;      // > 0: lists of pairs within 1 + skin kept until a rebuild (reach 1)
  int lanes;       // pass 2: lanes per particle (8, 16 or 32)
  int fblk;        // pass 2: 128-row blocks per CTA (1, 2 or 4)
  int dlanes;      // pass 1 over kept lists: lanes per particle (8, 16 or 32)
};
// Pass 1 and its densities (verlet: over the kept lists; marks: also the
// precursor marks, zeroed first over rows, the buffer's capacity).
// (lanes: lanes per particle of the kept-list pass, 8, 16 or 32)
void launch_density(const DevState& d, int nblk, int mode, int reach, bool verlet, bool marks,
                    size_t rows, cudaStream_t st, int lanes = 32);
// Precursor conversion after the force pass (marks: the FP32 pass 1 left its
// marks; else the cells are swept).
void launch_precursor(const DevState& d, int nblk, bool marks, cudaStream_t st);
// The kept lists of every particle (when this step rebuilds).
void launch_verlet_build(const DevState& d, int nblk, int reach, cudaStream_t st);
// Pass 2 (kept: pass 1 ran over the kept lists; rows: the capacity of the
// force sums, which the FP32 pass zeroes first, since its terms arrive by
// atomic add).
void launch_force(const DevState& d, int nblk, int mode, bool with_press, bool kept,
                  const PairTuning& tu, int form_mask, size_t rows, cudaStream_t st);
void launch_com(const DevState& d, int nblk, double* cm_out, uint32_t* cnt_out, cudaStream_t st);
// The sum of npair over rows [row0, row0 + n) into *out (device), zeroed first.
void launch_sum_pairs(const uint32_t* npair, int row0, int n, unsigned long long* out,
                      cudaStream_t st);
// The FP64 pass-2 kernels (plain and engine algorithm), launched by launch_force.
void launch_force_fp64(const DevState& d, int nblk, int mode, bool with_press, bool kept,
                       cudaStream_t st);

// kernels_chem.cu: one RandomChemEvent (LOCAL_CHEM_EVENT form) on replica 0.
// force: run regardless of Parameter::time >= beg_chem (fine-grained call).
struct ChemBuffers {
  ChemDev* chem;
  uint8_t* flags;      // [n_core * amp_cap] molecule inside the reaction cone
  int* chunk;          // [ceil(n_core * amp_cap / 1024)] flags per 1024-chunk
  uint32_t* targets;   // [2 * target_cap] head, tail storage rows
  uint32_t* draws;     // [25 * target_cap] MT draws of the placements
};
void launch_chem(const DevState& d, const ChemBuffers& b, int nblk, int n_core, int amp_cap,
                 bool force, cudaStream_t st);

// Observation of one step (kernels_integrate.cu): per row-block partial sums,
// per molecule values, then one record per due replica.
struct ObsPart {
  double v2[3];     // sum of v_k^2 over the block's rows
  long long pq[3];  // sum of press_i (the pair pass's 2^-26 fixed point)
  double ds2;       // sum of |delta_sumr|^2
  double dsol2;     // the same over rows whose upload index is >= amp_num
};
struct ObsBuffers {
  ObsPart* part;            // [row blocks]
  double* mvir;             // [molecules * 3] bonded virial per molecule
  double* mdif;             // [molecules] |mean delta_sumr of rows 4i..4i+3|^2
  idpd_observation* rec;    // [cap] records
  int* count;               // records written (may exceed cap: dropped)
  int cap;
  int period;
};
// Bonded virial per molecule; launched right after the bonded pass (before a
// reaction event adds molecules).
void launch_observe_bonds(const DevState& d, const ObsBuffers& b, int n_amp_tot,
                          const int* amp_rep, cudaStream_t st);
// Row sums, molecule diffusion and the records; launched after the step's
// last velocity change, before the step counter advances.
void launch_observe(const DevState& d, const ObsBuffers& b, int nblk, int n_amp_tot,
                    const int* amp_rep, int R, cudaStream_t st);
// Density profile and radial distribution of replica r (counts added to
// hist, int64 per bin).
void launch_density_profile(const DevState& d, int r, int row_off, int n, int axis, int nbins,
                            unsigned long long* hist, cudaStream_t st);
void launch_rdf(const DevState& d, int r, int row_off, int n, int nbins, double r_max, int m,
                unsigned long long* hist, cudaStream_t st);

// kernels_walks.cu: the FDPS multi-walk passes (buffers per handle).
struct WalkState;
WalkState* walk_create();
void walk_destroy(WalkState* s);
int walk_dispatch(WalkState* s, cudaStream_t st, const RepDev& R, const idpd_params& p, int kind,
                  int tag, int n_walk, const void* const* epi, const int32_t* n_epi,
                  const void* const* epj, const int32_t* n_epj, std::string& err);
int walk_retrieve(WalkState* s, int kind, int tag, int n_walk, const int32_t* ni,
                  void* const* result, std::string& err);

// kernels_integrate.cu
void launch_bonded_kick(const DevState& d, int nblk, bool kick, cudaStream_t st);
void launch_bonded_fine(const DevState& d, int n_amp_tot, const int* amp_rep, double* vir_part,
                        cudaStream_t st);
void launch_kick_only(const DevState& d, int nblk, cudaStream_t st);
void launch_fq_to_acc(const DevState& d, int nblk, double* press_out, cudaStream_t st);
void launch_cmdrift(const DevState& d, int nblk, int R, bool force_now, cudaStream_t st);
// skip (may be null): device flag that, when set, leaves the step counter
// unchanged (the reference breaks out of its loop before time++).
void launch_time_advance(const DevState& d, int R, cudaStream_t st, const int* skip = nullptr);
// The K-step loop graph: the count of steps, and the last node of each step.
void launch_loop_set(int* left, int n, cudaStream_t st);
void launch_loop_tail(cudaGraphConditionalHandle cond, int* left, const int* stop,
                      cudaStream_t st);
void launch_saru_test(int n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3, int draws,
                      uint32_t* out_u, float* out_n, cudaStream_t st);
void launch_aos_to_soa(const double* aos, double* x, double* y, double* z, int n, cudaStream_t st);
void launch_set_dynamics(const DevState& d, const double* pos, const double* vel,
                         const double* acc, int row0, int n, double box0, double box1,
                         double box2, bool kept, cudaStream_t st);
void launch_soa_to_aos(const double* x, const double* y, const double* z, const uint32_t* loc,
                       int row0, double* aos, int n, cudaStream_t st);
void launch_gather_u32x4(const uint32_t* a, const uint32_t* b, const uint32_t* c,
                         const uint32_t* e, const uint32_t* loc, int row0, uint32_t* out, int n,
                         cudaStream_t st);

}  // namespace idpd
