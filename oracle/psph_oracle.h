/*
 * CPU restatement of PersianSPH's per-step hot path: the parity ORACLE.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs may load it, and only as the checker or as the
 * timed CPU implementation of the reference algorithm; the GPU product never
 * calls it. It shares the boundary's plain-C structures (include/psph.h) so a
 * test can feed the same particles to both sides.
 *
 * Pinning: the restatement is checked against the unmodified reference built
 * here (oracle/build_ref.sh -> oracle/_ref/ref_driver) through the committed
 * fixtures in tests/golden/ (generated by tests/golden/make_golden.py).
 */
#ifndef PSPH_ORACLE_H
#define PSPH_ORACLE_H

#include "psph.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct psph_oracle psph_oracle;

/* initial != 0: Solve's set-up (InitialChecks, CellInitiate, ListGenerate).
 * grid / integ (may be NULL) continue from a saved state instead. */
psph_oracle* psph_oracle_create(const psph_config* cfg, const psph_particles* p, int initial,
                                const psph_grid* grid, const psph_integrator* integ);
void psph_oracle_destroy(psph_oracle* o);
const char* psph_oracle_error(const psph_oracle* o);

/* nsteps of Solve's loop body with nthreads OpenMP threads (1 = the reference's
 * deterministic Nproc=1 order). Returns a psph_status. */
int psph_oracle_step(psph_oracle* o, int64_t nsteps, int nthreads);

int64_t psph_oracle_num_particles(const psph_oracle* o);
int psph_oracle_download(const psph_oracle* o, psph_particles* out);
/* original index of each surviving particle */
int psph_oracle_original_index(const psph_oracle* o, int64_t* out);
int psph_oracle_get_grid(const psph_oracle* o, psph_grid* g);
int psph_oracle_get_integrator(const psph_oracle* o, psph_integrator* it);

/* Pair lists of the NEXT step's neighbour search from the current state, as
 * original indices (first, second): which 0 = SM, 1 = FSM, 2 = NSM, 3 = the
 * in-support subset of all three. Returns the count (<0 on error). */
int64_t psph_oracle_pairs(psph_oracle* o, int which, int64_t* buf, int64_t cap);

/* Per-particle magnitude of the sums behind the last step's acceleration and
 * density rate: |g| + |body force| + sum_j |m_j F_ij|, and sum_j |m_j (di/dj) v.gradW|.
 * Tests scale their per-particle tolerance by these. */
int psph_oracle_scales(const psph_oracle* o, double* a_scale, double* drho_scale);

/* A user InCon (which = PSPH_FLOW_IN) or OutCon (PSPH_FLOW_OUT) for an
 * in/out-flow domain, with psph_set_flow_profile's meaning; fn = NULL restores
 * the reference's default (the BC constants). */
int psph_oracle_set_flow_profile(psph_oracle* o, int which, psph_flow_fn fn, void* user);

/* Domain::GeneralBefore / GeneralAfter (psph_set_step_hooks' meaning): fn runs
 * after the neighbour search (PSPH_HOOK_BEFORE) and after the forces
 * (PSPH_HOOK_AFTER) of every step; inside it psph_oracle_download and
 * psph_oracle_patch read and write the particles. A non-zero return stops the
 * step with PSPH_ERR_STATE. */
typedef int (*psph_oracle_hook_fn)(psph_oracle* o, int where, void* user);
int psph_oracle_set_step_hooks(psph_oracle* o, psph_oracle_hook_fn fn, void* user, int where_mask);
int psph_oracle_patch(psph_oracle* o, const psph_particles* p);

/* In-support pairs CalcForce11 / CalcForce2233 evaluated (the pair-interaction
 * count of the metric), summed over the steps since create. */
int64_t psph_oracle_pair_count(const psph_oracle* o);

/* Wall time (s) of the phases of the last psph_oracle_step call: search,
 * wall interpolation, pair forces, update, relist; returns the count. */
int psph_oracle_phase_times(const psph_oracle* o, double* s, int cap);

#ifdef __cplusplus
}
#endif

#endif
