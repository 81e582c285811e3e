/*
 * persiansph-gb300 C ABI: the drop-in boundary for PersianSPH's per-step hot
 * path on one GB300 (sm_103a).
 *
 * The reference runs its hot path as methods of SPH::Domain called from
 * Domain::Solve (Source/Domain.cpp:1735-1797). This ABI replaces the body of
 * that loop (Source/Domain.cpp:1764-1792) and the set-up it relies on
 * (Source/Domain.cpp:1746-1751): a host wrapper keeps the Domain / Particle
 * API, packs the particles once into the structures below, and drives the
 * device through these calls. Plain C types only; no CUDA or torch types cross
 * the boundary (streams travel as void*).
 *
 * Conventions
 *  - Every call returns psph_status (0 = success). psph_last_error() gives the
 *    message; the C++ wrapper turns a non-zero status into the reference's
 *    `throw new Fatal(...)` (External/fatal.h:65).
 *  - Per-particle arrays are host arrays indexed by the particle's position in
 *    Domain::Particles at upload time ("original index"). Vectors are
 *    interleaved [3*i+d]; 3x3 tensors row-major [9*i+3*r+c].
 *  - One context = one Domain = one CUDA stream; calls on a context must come
 *    from one host thread at a time (the reference's Domain is not re-entrant
 *    either, Source/Domain.h:125).
 */
#ifndef PSPH_H
#define PSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3: psph_config gained the in/out-flow settings, psph_particles in_out */
#define PSPH_ABI_VERSION 3

typedef enum psph_status {
  PSPH_OK = 0,
  PSPH_ERR_INVALID_ARGUMENT = 1, /* bad enum/size/pointer; reference aborts or throws Fatal */
  PSPH_ERR_UNSUPPORTED = 2,      /* valid reference option outside this build (e.g. in/out-flow in FP32C) */
  PSPH_ERR_CUDA = 3,             /* a CUDA runtime call failed */
  PSPH_ERR_OUT_OF_MEMORY = 4,
  PSPH_ERR_NONFINITE = 5,        /* NaN/Inf found in an acceleration or density rate */
  PSPH_ERR_DT_COLLAPSE = 6,      /* "Too small time step" (Source/Domain.cpp:150-151) */
  PSPH_ERR_CFL = 7,              /* user dt above the CFL limit (Source/Domain.cpp:1731-1732) */
  PSPH_ERR_CELL_OVERFLOW = 8,    /* a cell holds more particles than the kernels stage */
  PSPH_ERR_NO_DEVICE = 9,        /* no CUDA device or not an sm_103 part */
  PSPH_ERR_STATE = 10,           /* call out of order (e.g. step before upload) */
  PSPH_ERR_NOT_FOUND = 11        /* DelParticles found no particle with the tag (Source/Domain.cpp:511) */
} psph_status;

/* Kernel_Set / Viscosity_Eq_Set / Gradient_Approach_Set (Source/Domain.h:38-40). */
enum { PSPH_QUBIC_SPLINE = 0, PSPH_QUINTIC = 1, PSPH_QUINTIC_SPLINE = 2 };
enum { PSPH_MORRIS = 0, PSPH_SHAO = 1, PSPH_INCOMPRESSIBLE_FULL = 2, PSPH_TAKEDA = 3 };
enum { PSPH_SQUARED_DENSITY = 0, PSPH_MULTIPLIED_DENSITY = 1 };
/* Domain::Scheme (Source/Domain.h:136). */
enum { PSPH_MVERLET = 0, PSPH_LEAPFROG = 1 };
/* Arithmetic form of the pair kernels. */
enum { PSPH_FP64 = 0, PSPH_FP32C = 1 };
/* Wall-pressure orientation (Source/Domain.cpp:1034-1053). REFERENCE reproduces
 * the reference's sign of the g.x_ij term, which depends on which particle its
 * neighbour search lists first; PHYSICAL always uses x_wall - x_fluid. */
enum { PSPH_WALLP_REFERENCE = 0, PSPH_WALLP_PHYSICAL = 1 };

/* Domain-level settings (public fields of SPH::Domain, Source/Domain.h:93-145). */
typedef struct psph_config {
  int32_t dimension;          /* Domain::Dimension: 2 or 3 */
  int32_t kernel_type;        /* PSPH_QUBIC_SPLINE ... */
  int32_t vis_eq;             /* PSPH_MORRIS ... */
  int32_t gradient_type;      /* PSPH_SQUARED_DENSITY ... */
  int32_t scheme;             /* PSPH_MVERLET or PSPH_LEAPFROG */
  int32_t periodic[3];        /* Domain::BC.Periodic */
  int32_t swi_type;           /* Domain::SWIType: fluid-soil interaction (CalcForce13) when fluid
                                 (Material 1) and soil (Material 3) share a domain: 0 seepage force,
                                 1 seepage + surface erosion, 2 seepage + pore pressure, 3 none
                                 (0, 1 and 3 also switch soil between saturated and dry weight) */
  int32_t shepard_step;       /* Particle::ShepardStep, uniform over particles (default 40) */
  int32_t precision;          /* PSPH_FP64 or PSPH_FP32C */
  int32_t wall_pressure_mode; /* PSPH_WALLP_REFERENCE or PSPH_WALLP_PHYSICAL */
  double gravity[3];          /* Domain::Gravity */
  double body_force[3];       /* constant acceleration added to free particles where the
                                 GeneralBefore hook runs (the 1-Poiseuille.cpp UserAcc pattern) */
  double xsph;                /* Domain::XSPH */
  double sqrt_h_a;            /* Domain::sqrt_h_a (default 0.0025) */
  double R;                   /* Domain::R: lattice half-spacing, pads periodic domains */
  double dom_max[3];          /* Domain::DomMax (default -1e11: no override) */
  double dom_min[3];          /* Domain::DomMin (default +1e11: no override) */
  double dt;                  /* Solve's dt argument: initial and maximum time step */
  double time;                /* Domain::Time at upload */
  int32_t fsi;                /* Domain::FSI: free solid particles take the pressure and velocity
                                 their free fluid neighbours interpolate (Source/Domain.cpp:1090-1160);
                                 fluid-solid pairs use CalcForce12 either way */
  int32_t in_out_flow;        /* Domain::BC.InOutFlow (Source/Domain.cpp:1327-1635): particles are
                                 given the in-flow state near -x (1), the out-flow state near +x (2),
                                 or both (3), and leaving particles are recycled to the in-flow; 0 none */
  int32_t mass_conservation;  /* BC.MassConservation: out-flow velocity scaled by |in| / |out| */
  int32_t reserved[5];        /* must be zero */
  double initial_dist;        /* Domain::InitialDist (spacing of the recycled in-flow lattice) */
  double bc_cellfac;          /* BC.cellfac: width of the in/out-flow zones in hmax (0: the reference's 3.9) */
  double in_v[3], in_density;   /* BC.inv, BC.inDensity: what the default InCon (InFlowCon) sets */
  double out_v[3], out_density; /* BC.outv, BC.outDensity: what the default OutCon (OutFlowCon) sets */
} psph_config;

/* Cell grid made by CellInitiate (Source/Domain.cpp:549-660). */
typedef struct psph_grid {
  double blpf[3];      /* Domain::BLPF, bottom-left-front corner after padding */
  double trpr[3];      /* Domain::TRPR */
  double cell_size[3]; /* Domain::CellSize */
  double dom_size[3];  /* Domain::DomSize (non-zero on periodic axes) */
  double hmax;         /* Domain::hmax */
  double rhomax;       /* Domain::rhomax */
  double cellfac;      /* Domain::Cellfac: 3 for the quintic spline, else 2 */
  int32_t cell_no[3];  /* Domain::CellNo, including the 2 ghost columns of a periodic axis */
  int32_t pad;
} psph_grid;

/* Time-integration state. The reference keeps FirstStep/ct/ShepardCounter per
 * particle, but every free particle advances them identically each step
 * (Source/Particle.cpp:189-274, :561-596), so they are held once per domain. */
typedef struct psph_integrator {
  double time;              /* Domain::Time */
  double deltat;            /* Domain::deltat */
  double deltatint;         /* Domain::deltatint (user dt) */
  double deltatmin;         /* Domain::deltatmin of the last step */
  int64_t steps;            /* steps taken since upload */
  int32_t first_step;       /* Particle::FirstStep */
  int32_t ct;               /* Particle::ct (Modified Verlet restart counter) */
  int32_t shepard_counter;  /* Particle::ShepardCounter */
  int32_t pad;
} psph_integrator;

/* Host view of the particles (SPH::Particle fields, Source/Particle.h:29-149).
 * Any pointer may be NULL: on upload the Particle-constructor default is used
 * (Source/Particle.cpp:25-117); on download the field is skipped. */
typedef struct psph_particles {
  int64_t n;
  /* int32 per particle */
  int32_t *id, *material, *is_free, *no_slip, *pres_eq, *shepard, *les, *vis_m, *fail;
  /* 3-vectors */
  double *x, *v, *va, *vb, *a, *nsv, *vxsph;
  /* scalars */
  double *density, *densitya, *densityb, *ddensity, *pressure, *mass, *h, *cs, *p0, *ref_density,
      *fpmassc, *alpha, *beta, *mu, *mu_ref, *t0, *bingham_m, *csmag, *ti, *tin, *ti_init_dist, *g_mod,
      *k_mod, *sigmay, *cohesion, *phi, *psi, *zwab, *sumden, *sumkernel, *shear_rate, *sbar;
  /* 3x3 tensors */
  double *sigma, *sigmaa, *sigmab, *shear_stress, *shear_stressa, *shear_stressb, *strain, *straina,
      *strainb, *strain_rate, *rotation_rate, *tir;
  /* Soil-water interaction of soil particles (Source/Particle.h:41-42, :110-121).
   * seepage_type: SeepageType (0 Darcy, 1 Kozeny-Carman, 2 Ergun, 3 Den Adel);
   * var_porosity: VarPorosity (porosity, k and k2 follow the volumetric strain);
   * is_sat: IsSat (on download, the saturation state after the last step);
   * n0, d, rho_f: initial porosity, grain size, fluid density RhoF;
   * k, k2: permeabilities, read on upload (an initial upload derives them from
   * n0 and d for SeepageType 1-3, as InitialChecks does), not written on download;
   * volume: V (default Mass/RefDensity, the Particle constructor's value);
   * s: S, the surface-erosion velocity derivative of the last step (download only). */
  int32_t *seepage_type, *var_porosity, *is_sat;
  double *n0, *k, *k2, *d, *rho_f, *volume, *s;
  /* Particle::InOut: 0, or 1 / 2 while the particle is in the in-flow / out-flow
   * state (config in_out_flow) */
  int32_t* in_out;
} psph_particles;

typedef struct psph_ctx psph_ctx;

/* Library / device probe. Returns PSPH_OK when an sm_103 device is usable. */
int psph_abi_version(void);
psph_status psph_device_check(int* device_count);

/* Domain construction: validates cfg (Domain ctor + selectors, Source/Domain.cpp:54-131). */
psph_status psph_create(const psph_config* cfg, psph_ctx** out);
void psph_destroy(psph_ctx* ctx);
const char* psph_last_error(const psph_ctx* ctx);
/* cudaStream_t to run on (NULL = the context's own stream). */
psph_status psph_set_stream(psph_ctx* ctx, void* cuda_stream);

/* Optional, before upload: continue with a saved grid / integrator state
 * instead of Solve's set-up. */
psph_status psph_set_grid(psph_ctx* ctx, const psph_grid* grid);
psph_status psph_set_integrator(psph_ctx* ctx, const psph_integrator* integ);

/* Copies particles to the device. With initial != 0 it also performs Solve's
 * set-up: InitialChecks (initial EOS pressure, Source/Domain.cpp:1662-1719),
 * CellInitiate (unless psph_set_grid was called) and TimestepCheck
 * (Source/Domain.cpp:1721-1733; returns PSPH_ERR_CFL like the reference throws). */
psph_status psph_upload(psph_ctx* ctx, const psph_particles* p, int initial);

/* Runs up to nsteps steps of Solve's loop body (Source/Domain.cpp:1764-1792),
 * stopping before a step when Domain::Time >= t_stop (Solve's `Time<tf` test).
 * *steps_done (may be NULL) receives the number of steps taken. */
psph_status psph_step(psph_ctx* ctx, int64_t nsteps, double t_stop, int64_t* steps_done);

/* Particles currently alive (CheckParticleLeave removes those leaving the grid). */
int64_t psph_num_particles(const psph_ctx* ctx);

/* Copies the current state into every non-NULL array of out (out->n must be at
 * least psph_num_particles). Particles come back in their original order with
 * deleted ones removed, as Array::DelItems leaves them (External/array.h:726). */
psph_status psph_download(psph_ctx* ctx, psph_particles* out);

/* Original index (position at upload) of each particle psph_download returns,
 * in the same order; out needs psph_num_particles entries. */
psph_status psph_original_index(psph_ctx* ctx, int64_t* out);

psph_status psph_get_grid(const psph_ctx* ctx, psph_grid* grid);
psph_status psph_get_integrator(const psph_ctx* ctx, psph_integrator* integ);

/* ---- In/out-flow profiles (Domain::InCon / OutCon, Source/Domain.h:128-129) ----
 * With in_out_flow set, InFlowBCFresh (Source/Domain.cpp:1594-1633) gives each
 * in-flow particle the velocity and density InCon returns for its position,
 * and each out-flow particle what OutCon returns (the velocity scaled by
 * MassConservation's InPart/OutPart ratio and taken only when out_v or that
 * ratio asks for it; the density only with out_density > 0). By default they
 * are the reference's InFlowCon / OutFlowCon, the constants in_v / in_density
 * and out_v / out_density of psph_config. A profile set here replaces one of
 * them: fn(x, v, density, user) gets the particle's position x[3] and writes
 * v[3] and *density (zero on entry). It runs on the calling thread inside
 * psph_step, once per in-flow (out-flow) particle per step, in BC.InPart order
 * (out-flow particles in original-index order). fn = NULL restores the
 * default. Contexts with in_out_flow != 0 only (PSPH_ERR_STATE otherwise). */
typedef void (*psph_flow_fn)(const double* x, double* v, double* density, void* user);
#define PSPH_FLOW_IN 1
#define PSPH_FLOW_OUT 2
psph_status psph_set_flow_profile(psph_ctx* ctx, int which, psph_flow_fn fn, void* user);

/* ---- Host hooks inside a step (Domain::GeneralBefore / GeneralAfter) ----------
 * The reference calls GeneralBefore after the neighbour search and
 * GeneralAfter after the forces and the time-step bound, both on the host with
 * the whole Domain in reach (Source/Domain.cpp:1767-1770). With a hook set,
 * psph_step launches each step in parts and calls fn(ctx, where, user) at
 * those points (where = PSPH_HOOK_BEFORE / PSPH_HOOK_AFTER, as selected by
 * where_mask). Inside fn the caller reads the particles with psph_download
 * (at PSPH_HOOK_BEFORE the accelerations are Gravity and the density rates
 * zero, as StartAcceleration left them; at PSPH_HOOK_AFTER this step's) and
 * writes changes back with psph_patch; psph_get_integrator gives Time. A
 * non-zero return from fn ends psph_step with PSPH_ERR_STATE. Each hook costs a
 * download and, when the hook patches, an upload of the particles: the slow
 * path for hooks that touch particles every step (a constant acceleration
 * belongs in psph_config.body_force instead). fn = NULL removes the hooks.
 * Single-domain contexts only. */
typedef int (*psph_hook_fn)(psph_ctx* ctx, int where, void* user);
#define PSPH_HOOK_BEFORE 1
#define PSPH_HOOK_AFTER 2
psph_status psph_set_step_hooks(psph_ctx* ctx, psph_hook_fn fn, void* user, int where_mask);

/* Writes particles back into a context: p holds psph_num_particles particles in
 * psph_download's order. The non-NULL arrays among the state fields (x, v, va,
 * vb, a, density, densitya, densityb, ddensity, pressure, mu when it varies
 * per particle, sigma, strain, shear_stress and their histories) replace the
 * device's values; the non-NULL per-particle parameters (mass, h, material
 * constants, flags, as psph_upload reads them) move a particle whose
 * parameters changed to the matching parameter set. Parameters that would
 * change what the step computes for the whole domain (a new material, a
 * different h where h is uniform, tensile instability, artificial viscosity,
 * strain rates or Shepard filtering where no particle had them, another EOS
 * where the fluid's is uniform) are refused with PSPH_ERR_UNSUPPORTED, as are
 * parameter changes in the FP32C form or in a fluid-soil / fluid-solid domain.
 * At PSPH_HOOK_BEFORE changed accelerations or density rates enter the step
 * as its starting values (FP64 form; the FP32C form refuses them). */
psph_status psph_patch(psph_ctx* ctx, const psph_particles* p);

/* Neighbour pairs of the current positions, as original indices, written as
 * (first, second) int64 couples in the orientation MainNeighbourSearch would
 * list them (Source/Domain.cpp:808-945). which = 0: every candidate pair
 * (SMPairs + FSMPairs + NSMPairs); which = 1: only pairs inside the kernel
 * support (r/h_ij <= Cellfac), the set CalcForce* works on. At most cap pairs
 * are written; *n_total receives the full count. */
psph_status psph_pairs_export(psph_ctx* ctx, int which, int64_t* pairs, int64_t cap, int64_t* n_total);

/* Device time of each phase of the last psph_step call, in ms: [0] cell sort +
 * reorder, [1] neighbour lists, [2] wall interpolation (and the FP32C copies),
 * [3] pair forces, [4] learned closure, [5] dt reduction, [6] update;
 * n_phases receives 7. Timing is recorded only when enabled. */
psph_status psph_enable_timing(psph_ctx* ctx, int enable);
psph_status psph_phase_times(const psph_ctx* ctx, double* ms, int cap, int* n_phases);
/* Number of kernel launches the last psph_step issued. */
int64_t psph_last_launch_count(const psph_ctx* ctx);
/* Steps since upload that ran the cell sort and the neighbour lists (every
 * step, unless the lists have a skin: psph_tuning.skin_permille). */
int64_t psph_list_rebuilds(psph_ctx* ctx);

/* psph_step(ctx, nsteps, +inf, steps_done) bracketed by CUDA events on the
 * context's stream; *device_ms receives the device time of the steps. */
psph_status psph_step_timed(psph_ctx* ctx, int64_t nsteps, double* device_ms, int64_t* steps_done);

/* ---- Launch tuning -----------------------------------------------------------
 * No counterpart in the reference (its loops run on OpenMP threads). The
 * launch shape of the FP32C pair kernels and the granularity of the cell sort
 * are chosen per context; psph_autotune measures the candidates on the
 * context's own workload. The cell grid itself stays the reference's
 * (CellInitiate): its cell size fixes the candidate pairs the FP64 form
 * reproduces; only the order inside a cell follows the split. */
typedef struct {
  int32_t pair_block;   /* threads per block of the FP32C pair kernels: 64, 128 or 256 */
  int32_t cell_split;   /* x-slabs per cell in the sort (1, 2 or 4): the neighbour-list walk
                           skips slabs out of reach */
  int32_t nlist_stage;  /* staging depth of the neighbour search: candidate positions each
                           block copies into shared memory (TMA bulk copies) before scanning
                           them, 2048, 3072 or 4096; 0 scans global memory. Applies with one
                           h everywhere and a non-periodic x axis. */
  int32_t skin_permille; /* FP32C form: neighbour lists with a skin of this many thousandths of the
                            support (0 to 150; 0, the default, lists every step). The lists then
                            hold every pair within (1 + skin) of the support, on cells at least
                            that wide, and the cell sort and the lists run again only when a
                            particle has moved half the skin (or left, or was patched); each step
                            still evaluates exactly the pairs inside the support. Domains without
                            a periodic axis and without Material 2; pair exports keep the
                            reference's cells. */
  double ms_per_step;   /* psph_autotune: device time per step of the chosen setting */
} psph_tuning;
psph_status psph_get_tuning(const psph_ctx* ctx, psph_tuning* out);
/* Applies a setting (the step graph is captured again at the next step). */
psph_status psph_set_tuning(psph_ctx* ctx, const psph_tuning* t);
/* Runs steps_per_trial timed steps (after one untimed step) with every
 * candidate setting and keeps the fastest; *chosen (if not NULL) receives it:
 * first every pair block x cell split, then, with those fixed, every staging
 * depth, then (FP32C) list skins of 50, 100 and 150 thousandths over at least
 * 24 steps each. The trial steps are real steps of the simulation: they
 * advance its time. */
psph_status psph_autotune(psph_ctx* ctx, int64_t steps_per_trial, psph_tuning* chosen);

/* ---- Snapshot output (WriteXDMF, Source/Domain.cpp:1869-2064) -----------------
 * The reference writes <key>.hdf5 (float32 datasets NP, Position, Velocity,
 * Acceleration, Tag, Pressure, Density, the three UserOutput properties under
 * OutputName[0..2], Mass, h, Sigma, Strain; Sigma and Strain as the six
 * components 00 01 02 11 12 22) and <key>.xmf. HDF5 is not linked here: the
 * same datasets, in the same order, types and values, go back to back into
 * <key>.bin (little endian; NP first), and <key>.xmf is the reference's XDMF
 * with each DataItem in Format="Binary" at its byte offset. names (may be
 * NULL, or hold NULL entries) are OutputName[0..2]; "Property1".."Property3"
 * by default. Single-domain contexts only. */
/* The next step psph_step takes writes a snapshot after its forces and before
 * its update, where Solve writes its output (Source/Domain.cpp:1773-1788), with
 * the default UserOutput properties (zeros, Source/Domain.cpp:28-33). The copy
 * to the host and the file writes overlap the steps that follow. */
psph_status psph_output_request(psph_ctx* ctx, const char* file_key, const char* const names[3]);
/* Writes a snapshot of the current state now (Solve's initial output,
 * Source/Domain.cpp:1752-1758), with the UserOutput properties prop1..prop3
 * (host arrays in psph_download order, or NULL for zeros); returns when the
 * files are written. */
psph_status psph_output_write(psph_ctx* ctx, const char* file_key, const char* const names[3], const double* prop1,
                              const double* prop2, const double* prop3);
/* Waits until every requested snapshot is written; reports a failed write. */
psph_status psph_output_flush(psph_ctx* ctx);

/* Pair-interactions evaluated since upload: unordered pairs {i,j}, at least
 * one free, r_ij <= Cellfac h_ij, summed over steps (the work CalcForce11 /
 * CalcForce2233 do in LastComputeAcceleration, Source/Domain.cpp:1238-1270). */
psph_status psph_pair_count(psph_ctx* ctx, uint64_t* pairs);

/* Pair export that allocates no device memory. It has no counterpart in the
 * reference: it serves callers that cannot call cudaMalloc where they need the
 * pairs (all device memory already handed to their own pool or another
 * framework's allocator, or a running loop that must not take cudaMalloc's
 * device-wide synchronisation). Same pairs as psph_pairs_export, written as
 * (first, second) int64 couples into the caller's DEVICE buffer pairs_device
 * (at most cap pairs, in sorted-particle order); *n_total (host) receives the
 * full count, also when cap < count (truncated output) or cap = 0 (count
 * only; pairs_device may then be NULL). Its scratch is one static device
 * array for at most PSPH_NOALLOC_MAX_PARTICLES particles (about 8 MB, kept by
 * every GPU that loads the library until exit); larger contexts, and exports
 * of more than PSPH_NOALLOC_MAX_PAIRS pairs (its offsets are 32-bit), get
 * PSPH_ERR_INVALID_ARGUMENT with nothing written. The first call on a device
 * looks up that array's device address (once per device, safe from several
 * threads): make it before any stream capture, and do not use the entry point
 * across a cudaDeviceReset. Calls share the array, so calls that overlap on
 * the GPU race. */
#define PSPH_NOALLOC_MAX_PARTICLES (1 << 20)
#define PSPH_NOALLOC_MAX_PAIRS 2147483647
psph_status psph_pairs_export_noalloc(psph_ctx* ctx, int which, int64_t* pairs_device, int64_t cap,
                                      int64_t* n_total);

/* ---- Ensembles -----------------------------------------------------------
 * Many independent domains advanced together, no counterpart in the
 * reference (whose Domain holds one simulation; an ensemble there is a loop
 * of processes, each running Solve). A batch context holds ninst instances,
 * each with its own particles, cell grid (CellInitiate per instance), time
 * step (AdaptiveTimeStep per instance) and stop time; every step runs one
 * set of kernel launches over all instances' particles. The instances share
 * the physics switches of psph_config (dimension, kernel, viscosity equation,
 * gradient type, scheme, precision, wall pressure mode, gravity, body force,
 * XSPH, sqrt_h_a, Shepard step); the per-particle parameters, R, the domain
 * bounds and dt may differ. Particle indices are per instance.
 * Each instance of a batch evolves exactly as a single-domain context fed the
 * same particles would (same pairs, same summation order per particle). */
psph_status psph_batch_create(const psph_config* cfgs, int ninst, psph_ctx** out);
int psph_batch_size(const psph_ctx* ctx);
/* parts[0..ninst): one particle set per instance. */
psph_status psph_batch_upload(psph_ctx* ctx, const psph_particles* parts, int initial);
/* Advances every instance until it has done nsteps steps or reached its stop
 * time t_stop[q] (NULL: no stop time); steps_done[q] (if not NULL) receives
 * the steps instance q made. */
psph_status psph_batch_step(psph_ctx* ctx, int64_t nsteps, const double* t_stop, int64_t* steps_done);
int64_t psph_batch_num_particles(const psph_ctx* ctx, int inst);
psph_status psph_batch_download(psph_ctx* ctx, int inst, psph_particles* out);
psph_status psph_batch_original_index(psph_ctx* ctx, int inst, int64_t* out);
psph_status psph_batch_get_grid(const psph_ctx* ctx, int inst, psph_grid* grid);
psph_status psph_batch_get_integrator(const psph_ctx* ctx, int inst, psph_integrator* integ);

/* ---- Learned closure -------------------------------------------------------
 * No counterpart in the reference. A small MLP predicts the eddy viscosity
 * that the LES option computes with the Smagorinsky model in Mat1
 * (Source/Particle.cpp:157-160: Mu = MuRef + RefDensity (CSmag h)^2 SBar).
 *
 * Inputs (raw features, per fluid particle with LES on, from the step's own
 * pair sums; StrainRate is the reference's fluid strain rate, twice the
 * symmetric velocity gradient D):
 *   [0] log(ShearRate h / Cs), ShearRate = sqrt(StrainRate:StrainRate / 2)
 *   [1] det(StrainRate) / (StrainRate:StrainRate)^(3/2)   (0 in 2D)
 *   [2] log(|vorticity| h / Cs)
 *   [3] Density / RefDensity
 *   [4] h / dx            (dx = the lattice spacing given to psph_closure_attach)
 *   [5] number of neighbours inside the kernel support
 * (logs of max(value, 1e-12); the rates are in units of the acoustic rate
 * Cs / h, so the features of one flow change little with the lattice). The network is 6 -> 64 -> 64 -> 64 -> 1 with
 * SiLU hidden layers; the three hidden layers run on the tensor cores
 * (tcgen05, BF16 weights and activations, FP32 accumulation); the output c =
 * softplus(z) gives the eddy viscosity nu_t = c h^2 ShearRate, and
 * Mu = MuRef + RefDensity nu_t. A particle whose features fall outside the
 * training range [lo, hi] uses the Smagorinsky term instead (counted), except
 * that rates below the range (fluid at rest, where nu_t vanishes with
 * ShearRate) are raised to its floor.
 *
 * Parameters (PSPH_MLP_NPARAMS floats, FP32 masters; W1..W3 are rounded to
 * BF16 when used): W1[64][6], b1[64], W2[64][64], b2[64], W3[64][64], b3[64],
 * w4[64], b4. Normalisation (PSPH_MLP_NNORM floats): mean[6], inv_std[6],
 * lo[6], hi[6]; the network sees (feature - mean) * inv_std. */
#define PSPH_MLP_INPUTS 6
#define PSPH_MLP_HIDDEN 64
#define PSPH_MLP_NPARAMS 8833
#define PSPH_MLP_NNORM 24
typedef struct psph_mlp psph_mlp;
/* Random initial weights (seeded); allocates on the current device. */
psph_status psph_mlp_create(uint64_t seed, psph_mlp** out);
void psph_mlp_destroy(psph_mlp* mlp);
const char* psph_mlp_last_error(const psph_mlp* mlp);
psph_status psph_mlp_set_params(psph_mlp* mlp, const float* params, const float* norm);
psph_status psph_mlp_get_params(const psph_mlp* mlp, float* params, float* norm);
/* Training set: x[n][6] raw features, y[n] target coefficients c. Sets the
 * normalisation (mean, 1/std, and the range [lo, hi] widened by 5%). */
psph_status psph_mlp_set_data(psph_mlp* mlp, const float* x, const float* y, int64_t n);
/* Per-sample loss weights w[n] of the training set (scaled to mean 1; NULL
 * drops them): loss = mean w (softplus(z) - y)^2. */
psph_status psph_mlp_set_weights(psph_mlp* mlp, const float* w);
/* Adam steps on minibatches of the training set (a new seeded permutation per
 * pass); loss = mean w (softplus(z) - y)^2. losses[k] (if not NULL) receives
 * the minibatch loss of step k. */
psph_status psph_mlp_train(psph_mlp* mlp, int64_t steps, int batch, float lr, uint64_t seed, float* losses);
/* Loss and gradient over (x, y) without changing the parameters. */
psph_status psph_mlp_loss_grad(psph_mlp* mlp, const float* x, const float* y, int64_t n, double* loss, float* grad);
/* Network output c for raw features x[n][6]: tensor_cores = 1 runs the
 * tcgen05 kernel used inside the step, 0 the same arithmetic on CUDA cores. */
psph_status psph_mlp_infer(psph_mlp* mlp, const float* x, int64_t n, float* c, int tensor_cores);
/* Puts the closure into the step of a context: every LES fluid particle then
 * takes its eddy viscosity from the network (copied at this call). After
 * psph_upload; dx is the lattice spacing of feature [4]. */
psph_status psph_closure_attach(psph_ctx* ctx, const psph_mlp* mlp, double dx);
/* Particles evaluated and particles that fell back to Smagorinsky, summed
 * over steps since attach. */
psph_status psph_closure_stats(psph_ctx* ctx, uint64_t* evaluated, uint64_t* fallbacks);
/* Raw features of the last step, out[6*i+k] for the particles of instance 0
 * in original order (zeros for particles without LES). */
psph_status psph_closure_features(psph_ctx* ctx, float* out);

/* Measurement helper with no counterpart in the reference: device FP64 FMA
 * throughput in TFLOP/s (an FMA counts 2), the roofline denominator of the
 * FP64 pair kernels. */
psph_status psph_probe_fp64_peak(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* PSPH_H */
