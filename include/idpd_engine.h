/*
 * idpd_engine.h - C ABI of the GB300 engine for the implicit-solvent MDPD
 * short-range particle step (kohnakagawa/implicit_dpd).
 *
 * Plain C: pointers, sizes and status codes only. Every entry point returns an
 * idpd_status; nothing aborts inside the library. Host arrays belong to the
 * caller and are copied in and out; device memory belongs to the handle.
 * Calls on one handle must be serialised by the caller; different handles are
 * independent. One CUDA stream per handle.
 *
 * Each entry point names the reference interface it replaces as
 * <file>:<line> inside the reference project.
 */
#ifndef IDPD_ENGINE_H
#define IDPD_ENGINE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IDPD_ABI_VERSION 1

typedef enum idpd_status {
  IDPD_OK = 0,
  IDPD_ERR_INVALID_ARG = 1, /* bad pointer, size, replica index or parameter  */
  IDPD_ERR_CAPACITY = 2,    /* particle / cell / neighbour capacity exceeded   */
  IDPD_ERR_CUDA = 3,        /* a CUDA runtime call failed                      */
  IDPD_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up              */
  IDPD_ERR_NONFINITE = 5,   /* NaN or Inf found in positions / forces          */
  IDPD_ERR_STATE = 6,       /* call order violated (e.g. force before upload)  */
  IDPD_ERR_NO_DEVICE = 7    /* no CUDA device is visible                       */
} idpd_status;

/* Bead properties (parameter.hpp:208-214). */
enum { IDPD_HYPHIL = 0, IDPD_HYPHOB = 1, IDPD_SOLVENT = 2, IDPD_PROP_NUM = 3 };

/* Conservative-force form of pass 2.
 *  MDPD:      CalcForceEpEpDPD default build (nbdf_calculator.hpp:119-123),
 *             density weight (1-r)^2 with hard cutoff 1 (nbdf_calculator.hpp:38-41).
 *  PAIRWISE:  the PAIRWISE_DPD build, a = 25 (nbdf_calculator.hpp:114-117).
 *  WARREN:    Warren's MDPD, A w_C + B (rho_i + rho_j) w_B with w_B = 1 - r/rd and
 *             density weight 15/(2 pi rd^3) (1 - r/rd)^2. Not in the reference;
 *             the dissipative and random terms stay the reference's. */
enum { IDPD_FORM_MDPD = 0, IDPD_FORM_PAIRWISE = 1, IDPD_FORM_WARREN = 2 };

/* Per-system physical parameters. Tables are the reference's static
 * coefficient tables after CalcInterCoef (parameter.hpp:138-186): cf_r is
 * already divided by sqrt(dt) and cf_g = cf_r_raw^2 / (2 kT). */
typedef struct idpd_params {
  double box[3];
  double dt;
  double cf_c[3][3];
  double cf_g[3][3];
  double cf_r[3][3];
  double cf_m[3][3][3];
  double cf_s;       /* bond coefficient, F = cf_s (1/r - 1/l0) d (parameter.hpp:713-716) */
  double cf_b;       /* bend coefficient (bdf_calculator.hpp:117-150)                    */
  double cf_b_rigid; /* bend coefficient of core molecules (bdf_calculator.hpp:77-86)    */
  double warren_a, warren_b, warren_rd; /* IDPD_FORM_WARREN only */
  uint32_t seed;     /* CalcForceEpEpDPD::m_seed (nbdf_calculator.hpp:65)   */
  uint32_t time;     /* Parameter::time of the next force pass (parameter.hpp:261) */
  int32_t form;      /* IDPD_FORM_* */
  int32_t reserved;
} idpd_params;

/* Inputs of Parameter::CalcInterCoef as run_param.txt gives them
 * (parameter.hpp:74-136; values already rounded through float like std::stof). */
typedef struct idpd_run_param {
  double box[3];
  double dt;
  double cf_r_upper[6]; /* upper triangle of cf_r, row major (parameter.hpp:29-38, 83-85) */
  double cf_s, cf_b, cf_b_rigid;
  double vbb, chi, kappa, rho_co;
} idpd_run_param;

/* Chemical-reaction parameters of one replica (Parameter members read by
 * ChemManager, parameter.hpp:230-243; amp_num/max_amp_num parameter.hpp:224,233). */
typedef struct idpd_chem_params {
  double p_thresld, eps;
  double influ_rad, influ_hei, influ_dep, influ_grd;
  uint32_t amp_num, max_amp_num;
} idpd_chem_params;

/* Derives idpd_params tables from run_param inputs exactly as
 * Parameter::CalcInterCoef (parameter.hpp:138-186) with the compile-time
 * constants of parameter.hpp:189-205. form/seed/time are left at zero. */
int idpd_derive_params(const idpd_run_param* rp, idpd_params* out);

/* ------------------------------------------------------------------------ */
/* Engine handle: device-resident state of one or more independent systems
 * ("replicas") advanced together. Replaces the FDPS ParticleSystem plus the
 * two Gather trees of src/main.cpp:93-132. */

typedef struct idpd_handle idpd_handle;

typedef struct idpd_config {
  int32_t n_replicas;      /* >= 1                                              */
  int32_t capacity;        /* max particles over all replicas (0 = auto at upload) */
  int32_t device;          /* CUDA device ordinal                               */
  int32_t flags;           /* IDPD_CFG_*                                        */
  int32_t sort_period;     /* steps between storage reorders by cell (0 = 100)  */
  int32_t reserved[3];
} idpd_config;

#define IDPD_CFG_FP64_PAIRS 0x1 /* plain FP64 pair kernels (baseline arm)       */
#define IDPD_CFG_TIMING 0x2     /* record per-kernel CUDA events                */
/* The engine's own algorithm (kept lists, each pair once, 64-bit fixed-point
 * sums) with FP64 pair arithmetic: the FP32 engine's denominator with the
 * algorithm held fixed. Cell reach 1 only; excludes IDPD_CFG_FP64_PAIRS. */
#define IDPD_CFG_FP64_KEPT 0x4
/* Plain graphs: idpd_step(h, K) launches one graph per step, and the step's
 * graph holds no conditional nodes (every gated kernel is launched and skips
 * itself). By default the K steps go to the device in one launch, a graph
 * whose conditional WHILE node repeats the captured step K times (between
 * storage reorders and observing steps), and the step's rarely needed work
 * (the cell and list rebuild, the drift removal) sits in conditional IF
 * nodes. Results are the same either way; profilers that cannot trace the
 * kernels of graphs with conditional nodes need the plain form. */
#define IDPD_CFG_PLAIN_GRAPHS 0x8

int idpd_create(const idpd_config* cfg, idpd_handle** out);
int idpd_destroy(idpd_handle* h);
/* Copies the last error message of the handle (or, when h is NULL, of the
 * last failed call without a handle on the calling thread) into buf, NUL
 * terminated. */
int idpd_last_error(const idpd_handle* h, char* buf, size_t len);

/* Parameters of one replica (the Parameter statics + CalcForceEpEpDPD::m_seed). */
int idpd_set_params(idpd_handle* h, int32_t replica, const idpd_params* p);
int idpd_get_params(const idpd_handle* h, int32_t replica, idpd_params* p);

/* FPDPD state of one replica, in FPDPD field order (ptcl_class.hpp:29-35):
 * pos/vel/acc are n x 3 doubles; id/prop/amp_id/unit n uint32 (amp_id and
 * unit 0xffffffff for solvent). Uploading replica r resets its particle
 * count to n; replicas are packed in replica order. delta_sumr is reset to 0. */
int idpd_upload_state(idpd_handle* h, int32_t replica, int32_t n, const double* pos,
                      const double* vel, const double* acc, const uint32_t* id,
                      const uint32_t* prop, const uint32_t* amp_id, const uint32_t* unit);
int idpd_num_particles(const idpd_handle* h, int32_t replica, int32_t* n);
/* Per-step exchange for a host that keeps the particle state (the FDPS
 * driver loop, src/main.cpp:166-184): overwrites pos/vel/acc of the rows of
 * an uploaded replica, in upload order, keeping ids, properties and the
 * topology. Positions outside [0, box] or non-finite values are rejected by
 * the device and reported by the next call (before the first pass after an
 * upload, they are checked on the host and the staged rows are replaced).
 * The arrays may also lie in device or managed memory: the kernels then read
 * them where they lie (before the first pass, they are copied to the host). */
int idpd_set_dynamics(idpd_handle* h, int32_t replica, const double* pos, const double* vel,
                      const double* acc);
/* Any pointer may be NULL to skip that field. Rows come back in the order
 * they were uploaded (new particles from chemistry appended). Buffers in
 * device or managed memory are written there by the kernels (or by copies,
 * before the first pass). */
int idpd_download_state(idpd_handle* h, int32_t replica, double* pos, double* vel, double* acc,
                        uint32_t* id, uint32_t* prop, uint32_t* amp_id, uint32_t* unit);
/* One MD step on host arrays: the reference's loop body (src/main.cpp:166-209)
 * with the particles' FPDPD pos/vel/acc (ptcl_class.hpp:29-31) kept in host
 * memory by the caller. The rows of the replica go in as idpd_set_dynamics,
 * every replica takes one step as idpd_step(h, 1), and the new pos/vel/acc
 * come back in place, in upload order, as idpd_download_state. The result is
 * that of the three calls bit for bit; the positions, final after the drift,
 * are copied back while the pair passes run, and the call synchronises once.
 * Not with the reaction enabled (IDPD_ERR_STATE: the reaction can add
 * particles during the step). The arrays may lie in device or managed memory,
 * as for idpd_set_dynamics and idpd_download_state. */
int idpd_step_host(idpd_handle* h, int32_t replica, double* pos, double* vel, double* acc);
/* Derived per-particle fields: density[3] (FPDPD::density), press[3]
 * (FPDPD::press), nei_cm_pos[2][3] (FPDPD::nei_cm_pos), delta_sumr[3]. */
int idpd_download_aux(idpd_handle* h, int32_t replica, double* density, double* press,
                      double* nei_cm_pos, double* delta_sumr);

/* Molecule topology of one replica: ForceBonded ctor (bdf_calculator.hpp:32-88):
 * glob_topol[amp*4+unit] = particle row, bend coefficient cf_b or cf_b_rigid for
 * the listed core molecules. Built from the uploaded amp_id/unit fields. */
int idpd_build_topology(idpd_handle* h, int32_t replica, int32_t n_amp, int32_t n_core,
                        const uint32_t* core_amp_id);

/* ---- fine-grained passes (all replicas at once) ------------------------- */

/* drift_and_predict (driftkick.hpp:6-27). */
int idpd_drift(idpd_handle* h);
/* dens_tree.calcForceAllAndWriteBack(CalcDensity()) (src/main.cpp:173;
 * nbdf_calculator.hpp:11-60; write-back ptcl_class.hpp:53-57), including the
 * neighbour centre-of-mass sums. */
int idpd_density(idpd_handle* h);
/* force_tree.calcForceAllAndWriteBack(CalcForceEpEpDPD()) (src/main.cpp:174;
 * nbdf_calculator.hpp:63-145; write-back ptcl_class.hpp:48-51): acc is
 * overwritten, press written. */
int idpd_force(idpd_handle* h);
/* ForceBonded::CalcListedForce (bdf_calculator.hpp:191-220): acc += bond and
 * bend forces. vir receives 3 doubles per replica (may be NULL). */
int idpd_bonded(idpd_handle* h, double* vir);
/* kick (driftkick.hpp:33-40). */
int idpd_kick(idpd_handle* h);
/* remove_cmdrift_global (driftkick.hpp:43-54), per replica. */
int idpd_remove_cmdrift(idpd_handle* h);

/* nsteps iterations of the main loop body of src/main.cpp:166-184 (drift,
 * density, force, bonded, kick, centre-of-mass drift removal every 100 steps,
 * time += 1) for every replica, captured once into a CUDA graph. The steps up
 * to the next storage reorder or observing step go to the device in one
 * launch (the graph's conditional WHILE node repeats the step, and ends the
 * loop after a step whose reaction event stopped the run); an observing step
 * is one launch, and with IDPD_CFG_PLAIN_GRAPHS every step is.
 * Per-particle press and nei_cm_pos are not produced by this path. */
int idpd_step(idpd_handle* h, int32_t nsteps);
/* Blocks until the handle's stream is idle; reports device-side errors. */
int idpd_sync(idpd_handle* h);

/* ---- chemical reaction (ChemManager, chemmanager.hpp:3-282) -------------- */
/* RandomChemEvent in its single-node LOCAL_CHEM_EVENT form (the form every
 * CHEM_MODE build uses, user_defs.h:6-8) on the device, for a handle with one
 * replica. Each event draws genrand_real1 of the ChemManager's MT19937 stream
 * for every molecule whose head lies inside a core's reaction cone, converts
 * the accepted ones into new 4-bead molecules beside them, appends the new
 * rows (ids, rows and molecule numbers continue the existing ones) and
 * extends the bonded topology with them. Decisions and the MT stream are
 * bit-exact with the reference for the same positions and core geometry. */
#define IDPD_CHEM_MAX_CORE 8
typedef struct idpd_chem_config {
  idpd_chem_params p;       /* p_thresld, eps, influ_*, max_amp_num; p.amp_num is
                               ignored: the molecules of idpd_build_topology count */
  uint32_t mt_seed;         /* ChemManager(seed): PS::MT::init_genrand (:176-180)   */
  uint32_t beg_chem;        /* first step with an event (Parameter::beg_chem,
                               parameter.hpp:254; main.cpp:187)                    */
  int32_t n_core;           /* core particles (Parameter::core_ptcl_id), <= 8        */
  uint32_t core_ptcl_id[IDPD_CHEM_MAX_CORE];
  int32_t reserve_amp;      /* molecules the handle makes room for (4 rows each)     */
  int32_t reserved[3];
} idpd_chem_config;

/* Enables (cfg != NULL) or disables (cfg == NULL) the event for replica 0.
 * While enabled, idpd_step runs one event per step after kick and the
 * centre-of-mass correction once Parameter::time >= beg_chem
 * (src/main.cpp:182-196); when amp_num reaches max_amp_num the step loop ends
 * after that step without advancing time, as the reference's loop breaks, and
 * further idpd_step calls return IDPD_ERR_STATE. */
int idpd_set_chem(idpd_handle* h, int32_t replica, const idpd_chem_config* cfg);
/* One RandomChemEvent on the current state, whatever the step counter
 * (chemmanager.hpp:244). *cont = 0 when amp_num reached max_amp_num (the
 * reference's false return), else 1. */
int idpd_chem_event(idpd_handle* h, int32_t* cont);
typedef struct idpd_chem_info {
  int32_t n_targets;        /* molecules converted by the last event                */
  int32_t events;           /* events run so far                                    */
  int32_t stopped;          /* amp_num reached max_amp_num                          */
  uint32_t amp_num;         /* Parameter::amp_num                                   */
  /* GetCorePos of the last event per core: core position, hydrophobic and
   * hydrophilic neighbour centres of mass (nei_cm_pos[Hyphob], [Hyphil]) */
  double core_raw[IDPD_CHEM_MAX_CORE][9];
  /* DetermineTargetIdWithCorePos of the last event per core: the unit
   * head-to-tail vector (membrane normal) and the projected core position,
   * what ChemManager::h2t_vecs() / core_poss_h() name (chemmanager.hpp:183-189;
   * the reference declares both arrays but never fills them) */
  int32_t n_core;
  int32_t reserved;
  double h2t[IDPD_CHEM_MAX_CORE][3];
  double core_h[IDPD_CHEM_MAX_CORE][3];
} idpd_chem_info;
/* State of the last event; targets (may be NULL) receives up to cap pairs of
 * (head, tail) rows of the converted molecules in upload order. */
int idpd_chem_get_info(idpd_handle* h, int32_t replica, idpd_chem_info* info, uint32_t* targets,
                       int32_t cap);

/* ---- precursor conversion (the reaction of the membrane-with-precursor
 * workload; the reference's own reaction is ChemManager above) -------------
 * Every step, after the force pass, each particle of property prop_from that
 * has a particle of property prop_near within the cutoff (the step's pair
 * set, r < 1) converts to prop_to when Saru(id, time, seed).u32() <
 * threshold (threshold = p * 2^32 for a probability p per step; the Saru
 * 3-seed constructor and u32() of saruprng.hpp:239-255, 322-333). Decisions
 * read the properties of the start of the step, are integer and bit-exact,
 * and take effect from the next step's pair passes. */
typedef struct idpd_precursor {
  uint32_t prop_from;   /* precursor property (IDPD_SOLVENT in that workload)  */
  uint32_t prop_near;   /* property whose presence within the cutoff triggers
                           the draw (IDPD_HYPHOB: a tail bead)                 */
  uint32_t prop_to;     /* property after the conversion (IDPD_HYPHIL: a head)  */
  uint32_t threshold;   /* converts when the draw is below it                   */
  uint32_t seed;        /* third Saru seed                                       */
  int32_t enabled;
  int32_t reserved[2];
} idpd_precursor;
/* cfg NULL or enabled 0 switches the conversion off for that replica. */
int idpd_set_precursor(idpd_handle* h, int32_t replica, const idpd_precursor* cfg);
/* Conversions of the replica since its conversion was last set. */
int idpd_precursor_count(idpd_handle* h, int32_t replica, uint64_t* conversions);

/* ---- observables (Observer, observer.hpp:82-178) ---------------------------- */
/* One macro observation of a replica, taken at the end of a step whose
 * Parameter::time is a multiple of the observation period (Parameter::step_mac,
 * src/main.cpp:198-205), after the kick, the centre-of-mass correction and the
 * reaction event, from the same quantities the reference's Observer reads. */
typedef struct idpd_observation {
  uint32_t time;            /* Parameter::time of the step                        */
  int32_t replica;
  int32_t n;                /* particles                                          */
  int32_t n_amp;            /* molecules (Parameter::amp_num, Observer::NumAmp)   */
  double kin_temp[4];       /* KineticTempera: <vx^2>, <vy^2>, <vz^2>, their mean   */
  double pressure[3];       /* Pressure: (sum_i press_i / 2 + sum_i v_i^2 +
                               bonded_vir / 2) / volume                             */
  double diffusion[3];      /* Diffusion: D_ptcl, D_lipid, D_sol (mean squared
                               delta_sumr of particles, of molecule centres over
                               rows 4i..4i+3, of rows from amp_num on over sol_num) */
  double pair_virial[3];    /* sum_i press_i of the step's pair pass               */
  double bonded_virial[3];  /* the step's ForceBonded virial                       */
} idpd_observation;

/* period > 0: every step whose Parameter::time % period == 0 records one
 * idpd_observation per replica into a device buffer of `capacity` records
 * (the pair pass of those steps also sums the per-particle virial); period 0
 * switches observation off. */
int idpd_set_observe(idpd_handle* h, int32_t period, int32_t capacity);
/* Moves up to max recorded observations (oldest first) into out; *n receives
 * the count. IDPD_ERR_CAPACITY when records were dropped because the buffer
 * was full (the records that fit are still returned). */
int idpd_get_observations(idpd_handle* h, idpd_observation* out, int32_t max, int32_t* n);

/* Number density profile of replica r along axis (0, 1, 2) in nbins slabs,
 * per particle property: out[bin * 3 + prop] = particles / slab volume. */
int idpd_density_profile(idpd_handle* h, int32_t replica, int32_t axis, int32_t nbins,
                         double* out);
/* Radial distribution function of replica r over all particle pairs, nbins
 * (<= 1024) shells up to r_max (0 < r_max <= 2; every box side >=
 * 2 ceil(r_max) + 1): out[k] = g(r) of shell k. */
int idpd_rdf(idpd_handle* h, int32_t replica, int32_t nbins, double r_max, double* out);

/* ---- FDPS multi-walk interface (f_calculator_gpu.cuh:9-21) ---------------- */
/* The interaction groups ("walks") FDPS hands to a GPU force kernel: i
 * particles and the j particles it gathered for them (positions already
 * image-shifted). The structs have the field order and layout of the
 * reference's EPI/EPJ/RESULT types (ptcl_class.hpp:5-174), so arrays of those
 * types can be passed as they are. Pass 1 (kind IDPD_WALK_DENSITY) follows
 * CalcDensity (nbdf_calculator.hpp:11-60), pass 2 (IDPD_WALK_FORCE)
 * CalcForceEpEpDPD (:63-147) with replica 0's tables, seed and step counter.
 * Pair decisions are taken on the FP64 positions as the reference takes them;
 * pair terms are FP32 with 64-bit fixed-point sums. */
typedef struct idpd_epi_density { uint32_t prop; double pos[3]; } idpd_epi_density;
typedef struct idpd_epj_density { uint32_t prop; double pos[3]; } idpd_epj_density;
typedef struct idpd_result_density {
  double dens[3];
  double nei_pos_sum[2][3];
  uint32_t nei_cnt[2];
} idpd_result_density;
typedef struct idpd_epi_dpd {
  uint32_t id, prop;
  double pos[3], vel[3], dens[3];
} idpd_epi_dpd;
typedef struct idpd_epj_dpd {
  uint32_t id, prop, amp_id, unit;
  double pos[3], vel[3], dens[3];
} idpd_epj_dpd;
typedef struct idpd_result_dpd { double acc[3], press[3]; } idpd_result_dpd;
enum { IDPD_WALK_DENSITY = 0, IDPD_WALK_FORCE = 1 };

/* DispatchKernel: copies the walks to the device and starts the pass; returns
 * without waiting. epi[w] / epj[w] point to n_epi[w] / n_epj[w] structs of the
 * kind's EPI / EPJ type. One dispatch per kind may be in flight; tag is kept
 * for the matching retrieve. */
int idpd_dispatch_walks(idpd_handle* h, int32_t kind, int32_t tag, int32_t n_walk,
                        const void* const* epi, const int32_t* n_epi, const void* const* epj,
                        const int32_t* n_epj);
/* RetrieveKernel: waits for the dispatch with this kind and tag and writes
 * (does not add) the results of walk w's ni[w] i particles to result[w]. */
int idpd_retrieve_walks(idpd_handle* h, int32_t kind, int32_t tag, int32_t n_walk,
                        const int32_t* ni, void* const* result);

/* ---- on-disk formats (host only; no device needed) ------------------------ */
/* run_param.txt as Parameter::LoadParam reads it (parameter.hpp:352-387,
 * tags of MatchingTagValues :74-136): one "tag value ..." per line, ';'
 * starts a comment; reals pass through std::stof (float rounding), integers
 * through std::stoi. influ_vol + upside_rad, when given, set influ_grd and
 * influ_rad (CalcInfluGrdAndRad :42-56); otherwise influ_vol follows from
 * them (CalcInfluVol :58-72). The physics and run tags are required as in the
 * reference (IDPD_ERR_INVALID_ARG names the missing tag); the reaction tags
 * are optional here (has_chem = 0 when any is missing). */
typedef struct idpd_run_file {
  idpd_run_param rp;        /* box_leng, dt, cf_r, cf_s, cf_b, cf_b_rigid, vbb (0.1 when
                               absent), chi, kappa, rho_co                             */
  uint32_t init_amp_num, sol_num, all_time, step_mic, step_mac;
  int32_t has_chem;
  idpd_chem_params chem;    /* amp_num = init_amp_num                                  */
  double influ_vol, upside_rad;
  int32_t n_core;           /* core_amp_id entries (at most IDPD_CHEM_MAX_CORE kept)   */
  uint32_t core_amp_id[IDPD_CHEM_MAX_CORE];
} idpd_run_file;
int idpd_read_run_param(const char* path, idpd_run_file* out);

/* init_config.xyz / traject.xyz / fin_config.xyz (io_util.hpp:26-31,95-129;
 * rows of FPDPD::writeAscii / readAscii, ptcl_class.hpp:60-86): "<n>", "time
 * <t>", then per particle: type letter, pos, id, prop, amp_id, unit, vel,
 * vel_buf, acc, reals printed with %.15g. idpd_read_xyz reads at most cap rows
 * (IDPD_ERR_CAPACITY beyond) and checks the header and the row count; any
 * output pointer may be NULL. idpd_write_xyz appends a frame when append != 0
 * (traject.xyz); vel_buf NULL writes vel in its place. */
int idpd_read_xyz(const char* path, int32_t cap, int32_t* n, uint32_t* time, double* pos,
                  double* vel, double* vel_buf, double* acc, uint32_t* id, uint32_t* prop,
                  uint32_t* amp_id, uint32_t* unit);
int idpd_write_xyz(const char* path, int32_t append, uint32_t time, int32_t n, const double* pos,
                   const double* vel, const double* vel_buf, const double* acc,
                   const uint32_t* id, const uint32_t* prop, const uint32_t* amp_id,
                   const uint32_t* unit);

/* ---- asynchronous trajectory frames --------------------------------------
 * Observer::Trajectory (observer.hpp:295-305) writes traject.xyz frames with
 * io_util::WriteXYZForm (io_util.hpp:26-31) from the host particle system.
 * idpd_dump_xyz_async queues one such frame of replica `replica`'s current
 * state without stopping the step loop: the rows are gathered in upload
 * order on the handle's stream (so the frame is the state after every call
 * queued before it), copied to pinned host memory on a second stream, and a
 * host thread writes the frame (the idpd_write_xyz format, vel_buf = vel)
 * while later steps run. One frame is in flight at a time: a second call
 * first waits for the previous frame to be written. idpd_dump_wait blocks
 * until the queued frame is on disk and returns the status of the first
 * frame that failed since the last wait. */
int idpd_dump_xyz_async(idpd_handle* h, int32_t replica, const char* path, int32_t append);
int idpd_dump_wait(idpd_handle* h);

/* ---- tuning --------------------------------------------------------------- */
/* Launch and cell-grid shape of the pair passes. Every reach and launch shape
 * gives the same results bit for bit (all pair sums are fixed point); only
 * speed changes. */
typedef struct idpd_tuning {
  int32_t reach;        /* 1: cells >= rc, 27-cell stencil; 2: cells >= rc/2, 125 cells */
  float skin;           /* > 0: keep each particle's list of pairs within rc + skin and
                           rebuild cells and lists only when some particle has moved
                           more than skin / 2 (cells >= (rc + skin) / reach; every box
                           side >= 3 (rc + skin)). Pair sets stay exact; sums differ
                           from skin 0 only by FP32 rounding of the cell-local
                           coordinates. 0: cells and lists every step. */
  int32_t pair_lanes;   /* pass 2: lanes per particle, 4, 8, 16 or 32 (0: 16)     */
  int32_t pair_blocks;  /* pass 2: 128-row blocks per CTA, 1, 2 or 4 (0: 1)        */
  int32_t density_lanes; /* pass 1 over kept lists: lanes per particle, 4, 8, 16 or
                            32 (0: 32); fewer suit short lists (liquids)          */
  int32_t reserved[3];
} idpd_tuning;
int idpd_set_tuning(idpd_handle* h, const idpd_tuning* t);
int idpd_get_tuning(const idpd_handle* h, idpd_tuning* t);
/* Steps that rebuilt the cells and the kept lists since the lists were last
 * (re)allocated; 0 while the skin is 0. */
int idpd_list_rebuilds(idpd_handle* h, uint64_t* rebuilds);
/* Ordered pairs within the cutoff (r < 1, i != j, the pair set of
 * CalcForceEpEpDPD, nbdf_calculator.hpp:84-88) of replica `replica`, counted
 * exactly by the last density pass (the last step's, or idpd_density's): the
 * sum over particles of n_p, the pairs per particle of the pair passes'
 * roofline. 0 before the first density pass. */
int idpd_pair_count(idpd_handle* h, int32_t replica, uint64_t* ordered_pairs);

/* ---- timing -------------------------------------------------------------- */
/* Elapsed milliseconds of the last idpd_step call measured with CUDA events
 * on the handle's stream. */
int idpd_last_step_ms(const idpd_handle* h, float* ms);
/* Per-kernel event timing of one un-graphed step (IDPD_CFG_TIMING): names is a
 * '\n'-separated list, ms one entry per name. */
int idpd_profile_step(idpd_handle* h, char* names, size_t names_len, float* ms, int32_t max_k,
                      int32_t* n_k);

/* ---- Saru (saruprng.hpp:83-445) on the device ----------------------------- */
/* out[k] = k-th u32() of Saru(s1[i], s2[i], s3[i]) for k < draws, i < n
 * (row-major n x draws). */
int idpd_saru_u32(int32_t n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                  int32_t draws, uint32_t* out);
/* FP32 Box-Muller normal of Saru(s1,s2,s3).nrml() as the pair kernel computes it. */
int idpd_saru_nrml_f32(int32_t n, const uint32_t* s1, const uint32_t* s2, const uint32_t* s3,
                       float* out);

/* ---- cell list (the FDPS gather replacement) ----------------------------- */
/* Cell index per particle row and the stable cell-sorted order of the rows
 * for replica `replica` on the handle's search grid: floor(box / (1 + skin))
 * * reach cells per axis (idpd_set_tuning; floor(box) cells of the pair
 * cutoff 1.0 at the default reach 1, skin 0). perm[k] = row at sorted
 * position k. */
int idpd_cell_order(idpd_handle* h, int32_t replica, uint32_t* cell_of_row, uint32_t* perm);

/* ---- cell order without allocation ---------------------------------------
 * No counterpart in the reference. A cell index per row and the stable
 * cell-sorted order of the rows, on a grid of floor(box) cells per axis (cells
 * of the pair cutoff 1.0), for rows the caller already holds on the device,
 * computed without allocating any device memory. This is idpd_cell_order's
 * result at the engine's default tuning (cell reach 1, skin 0) only; other
 * tunings give idpd_cell_order other grids. It is meant for callers that
 * cannot call cudaMalloc: a host MD code whose own memory pool
 * owns the device budget, or a step loop that must not pay the device-wide
 * synchronisation that cudaMalloc / cudaFree can cause.
 *
 * Its scratch is one static device array of IDPD_NOALLOC_SCRATCH_BYTES
 * (about 8 MiB), which every GPU that loads this library holds until the
 * process exits. Limits: n <= IDPD_NOALLOC_MAX_ROWS and
 * floor(box[0]) * floor(box[1]) * floor(box[2]) <= IDPD_NOALLOC_MAX_CELLS;
 * larger inputs return IDPD_ERR_CAPACITY with a message.
 *
 *   pos          device, n rows of x y z (FP64) inside [0, box)
 *   box          host, the three box sides, each >= 1.0
 *   cell_of_row  device out, n cell indices ((cz ny + cy) nx + cx)
 *   perm         device out, perm[k] = row at sorted position k
 *   stream       cudaStream_t to queue the work on (NULL: default stream)
 *
 * The call queues its work and returns; the outputs are complete when the
 * stream reaches that point. Every call looks the scratch address up in the
 * context current on the calling thread (cudaGetSymbolAddress, which
 * allocates nothing), so switching contexts or resetting the device between
 * calls is safe. The first call on each device also loads the library's
 * device code there (set-up): make that first call before any stream
 * capture. All calls share the one array, which keeps the
 * last call's contents, so calls that overlap on the GPU (other streams,
 * other threads) race and corrupt each other's results: serialise them.
 * Errors are read with idpd_last_error(NULL, ...). */
#define IDPD_NOALLOC_MAX_ROWS (1 << 20)
#define IDPD_NOALLOC_MAX_CELLS (1 << 19)
#define IDPD_NOALLOC_SCRATCH_BYTES 8389888
int idpd_cell_order_noalloc(const double* pos, int32_t n, const double* box,
                            uint32_t* cell_of_row, uint32_t* perm, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* IDPD_ENGINE_H */
