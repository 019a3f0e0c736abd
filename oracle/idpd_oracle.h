/*
 * CPU oracle for the implicit_dpd short-range particle step.
 *
 * TEST INFRASTRUCTURE ONLY. A plain-C, FP64 restatement of the reference's
 * hot-path algorithms, used by the tests, by __graft_entry__.smoke() and by
 * bench.py's CPU-baseline leg as the checker. The product never links it.
 *
 * Every FP64 expression is evaluated in the reference's operation order
 * (built with -ffp-contract=off), and j particles are visited in the order of
 * the reference harness in oracle/ref: cells of side >= 1.2 (search_rad,
 * parameter.hpp:196), 27 neighbour cells dz-major from -1 to +1, rows
 * ascending within a cell. Parity against the reference itself is pinned by
 * the golden vectors in tests/golden, generated by tests/golden/make_golden.py
 * from the reference headers compiled unmodified (oracle/ref/ref_harness.cpp).
 */
#ifndef IDPD_ORACLE_H
#define IDPD_ORACLE_H

#include <stdint.h>
#include "idpd_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Saru (saruprng.hpp:83-445) */
void orc_saru_u32(uint32_t s1, uint32_t s2, uint32_t s3, int32_t count, uint32_t* out);
double orc_saru_nrml(uint32_t s1, uint32_t s2, uint32_t s3);

/* MT19937 (mt19937ar, the generator behind FDPS PS::MT) */
typedef struct orc_mt {
  uint32_t mt[624];
  int32_t mti;
} orc_mt;
void orc_mt_seed(orc_mt* g, uint32_t seed);
uint32_t orc_mt_u32(orc_mt* g);
double orc_mt_real1(orc_mt* g);
double orc_mt_real3(orc_mt* g);
void orc_mt_draws(uint32_t seed, int32_t n, uint32_t* out);

/* Parameter::CalcInterCoef (parameter.hpp:138-186) */
int orc_derive_params(const idpd_run_param* rp, idpd_params* out);

/* Cells of side >= r_cell: returns the number of cells, or -1 if fewer than 3
 * per axis. cell_of[n]; start[ncell+1]; members[n] (rows ascending per cell). */
int32_t orc_cells(int32_t n, const double* pos, const double* box, double r_cell, int32_t* nc,
                  int32_t* cell_of, int32_t* start, int32_t* members);

/* Pass 1 + write-back: dens[3n]; nei_cm[6n] (hydrophilic xyz, hydrophobic
 * xyz, already divided by the counts as FPDPD::copyFromForce does);
 * nei_cnt[2n]. nei_cm / nei_cnt may be NULL. */
int orc_density(const idpd_params* p, int32_t n, const double* pos, const uint32_t* prop,
                double* dens, double* nei_cm, uint32_t* nei_cnt, int32_t nthreads);

/* Pass 2 + write-back: acc[3n] overwritten, press[3n] written (may be NULL). */
int orc_force(const idpd_params* p, int32_t n, const double* pos, const double* vel,
              const uint32_t* id, const uint32_t* prop, const double* dens, double* acc,
              double* press, int32_t nthreads);

/* ForceBonded: topology glob_topol[4*n_amp] and bend coefficients, from
 * amp_id/unit (bdf_calculator.hpp:61-88). Returns 0 or -1 on a bad row. */
int orc_build_topology(int32_t n, const uint32_t* amp_id, const uint32_t* unit, int32_t n_amp,
                       int32_t n_core, const uint32_t* core_amp_id, double cf_b, double cf_b_rigid,
                       uint32_t* topol, double* cf_bend);
/* CalcListedForce (bdf_calculator.hpp:153-220), serial order: acc += F. */
void orc_bonded(const idpd_params* p, int32_t n_amp, const uint32_t* topol, const double* cf_bend,
                const double* pos, double* acc, double* vir);

/* drift_and_predict / kick / remove_cmdrift_global (driftkick.hpp:6-54). */
void orc_drift(const idpd_params* p, int32_t n, double* pos, double* vel, double* vel_buf,
               const double* acc, double* dsr);
void orc_kick(double dt, int32_t n, double* vel, const double* vel_buf, const double* acc);
void orc_remove_cmdrift(int32_t n, double* vel);

/* One main-loop iteration (src/main.cpp:166-184) without chemistry/observers.
 * state arrays as above; vel_buf scratch [3n]; p->time is advanced. */
int orc_md_step(idpd_params* p, int32_t n, double* pos, double* vel, double* vel_buf, double* acc,
                double* dsr, const uint32_t* id, const uint32_t* prop, int32_t n_amp,
                const uint32_t* topol, const double* cf_bend, double* dens, double* press,
                double* bonded_vir, int32_t nthreads);

/* Chemistry (chemmanager.hpp): one single-node RandomChemEvent with
 * LOCAL_CHEM_EVENT. */
/* State arrays have room for n_cap rows; new particles are appended, *n is
 * updated, and *amp_num_out receives the new amphiphile count. Returns 1 to
 * continue, 0 to stop (amp_num >= max_amp_num), -1 on capacity overflow.
 * nei_cm[6n] is the hydrophilic/hydrophobic neighbour centre of mass. */
int orc_chem_event(const idpd_params* p, const idpd_chem_params* cp, orc_mt* g, int32_t* n,
                   int32_t n_cap, double* pos, double* vel, double* vel_buf, double* acc,
                   double* dsr, uint32_t* id, uint32_t* prop, uint32_t* amp_id, uint32_t* unit,
                   const double* nei_cm, const uint32_t* topol, int32_t n_core,
                   const uint32_t* core_ptcl_id, uint32_t* amp_num_out, uint32_t* targets_out,
                   int32_t* n_targets_out);

/* All ordered pairs (i, j), i != j, within rc under the minimum image
 * (test/nearlist/near_list.cpp:69-92). Returns the count; writes at most cap. */
/* The precursor conversion of the membrane-with-precursor workload (no
 * reference function: the engine's idpd_precursor): every i with
 * prop[i] == from and some j != i with prop[j] == near within r < 1 (the
 * FP64 pair expression of pass 1) converts to `to` when the Saru(id_i, time,
 * seed) u32 draw is below threshold. Decisions read the properties on entry;
 * prop is updated in place. Returns the number of conversions, -1 when the
 * box is too small for the cell grid. */
int64_t orc_precursor(const idpd_params* p, int32_t n, const double* pos, const uint32_t* id,
                      uint32_t* prop, uint32_t time, uint32_t from, uint32_t near, uint32_t to,
                      uint32_t threshold, uint32_t seed, int32_t nthreads);

int64_t orc_pair_count(const idpd_params* p, int32_t n, const double* pos, int32_t nthreads);
int64_t orc_pairs_naive(int32_t n, const double* pos, const double* box, double rc,
                        uint32_t* pi, uint32_t* pj, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
