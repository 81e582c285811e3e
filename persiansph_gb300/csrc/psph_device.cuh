// Device state and kernel entry points of the GB300 hot path.
#pragma once

#include "psph_common.cuh"

namespace psph {

// Persistent per-particle arrays (reordered by the cell sort each step).
struct Persist {
  double4_32a* X4;   // x, y, z, Density
  double4_32a* V4;   // vx, vy, vz, Pressure
  double4_32a* H4;   // leapfrog: va, Densitya | Modified Verlet: vb, Densityb
  double4_32a* H4b;  // leapfrog: vb, Densityb (wall vb is read by the soil pair force) | MVerlet: null
  int* cls;      // class index
  int* orig;     // original particle index
  int* io;       // in/out-flow state (Particle::InOut: 0, 1 in-flow, 2 out-flow); null without the boundary
  double* mu;    // dynamic viscosity (LES / Bingham); null when constant per class
  // soil / solid tensors (9 doubles per particle, row-major); null without solids
  double* sigma;
  double* sigma_h;   // leapfrog Sigmaa | MVerlet Sigmab
  double* strain;
  double* strain_h;  // leapfrog Straina | MVerlet Strainb
  double* shear;     // ShearStress (solids, Material 2)
  double* shear_h;   // leapfrog ShearStressa | MVerlet ShearStressb
  double* tir;       // TIR (wall values persist between updates, as in the reference)
};

// Per-step arrays (sorted order of the current step; not reordered).
struct Scratch {
  int* key;        // cell key per particle (pre-sort order)
  int* count;      // ncells + 2 counters
  int* start;      // ncells + 3 exclusive prefix: cell c's particles are [start[c], start[c+1])
  int* sstart;     // ncells * xsub + 3 exclusive prefix over the x-slabs of the cells (xsub > 1)
  int* tmp_perm;
  int* perm;
  int* cellid;     // cell of each sorted particle (orphan/dead: -1)
  int* block_sums;
  // per-step derived / outputs
  float4* OFF32;     // (position - cell origin, h) in FP32, written by the reorder
  float4* OFFREF;    // with a skin: the position at the last rebuild in FP32 (displacements are measured from it)
  int* refcell;      // with a skin: each particle's cell in the reference's grid (x | y << 10 | z << 20),
                     // for the wall pressure's pair orientation
  int* nl;           // per-step neighbour lists, entry k of particle i at nl[k*ncap + i]:
                     // index | cell-offset code << 26
  int* nl_count;     // list length, or -1 when it exceeded the capacity (scan instead)
  float4* V32;       // FP32C form: (v, pressure)
  float4* D32;       // FP32C form: (1/density, pressure/density^2, sound speed, density)
  float4* SIG32;     // FP32C solids: symmetric Sigma, 2 per particle (00 01 02 11 | 12 22 - -)
  float4* TIR32;     // FP32C solids with TI: symmetric TIR, same layout
  float4* VB32;      // FP32C solids: wall history velocity (MVerlet vb / leapfrog vb)
  float4* V32LO;     // FP32C: v - (float)v, the low-order part of the velocity (fluids: .w = the
                     // particle's class index as int bits, loaded with it by the pair kernel)
  float* MU32;       // FP32C, per-particle viscosity (LES / Bingham): FP32 copy of Persist::mu
  float4* NSV32;     // FP32C: wall no-slip velocity in FP32
  double4_32a* D4;   // seen by partners: (1/density, pressure/density^2, sound speed, density);
                     // a wall's density is the inverse EOS of its interpolated pressure
  double4_32a* A4;       // ax, ay, az, dDensity
  // FP64 once-per-pair form: a partner's terms of a pair, in the partner's own
  // list slot (nl_index layout): (a, dDensity) and (ZWab, SumDen)
  double4_32a* half4;
  double2* half2;
  int* half_stamp;       // instance step + 1 when the slot was written this step
  double* zwab;
  double* s_acc;         // SWIType 1: Particle::S, the surface-erosion velocity derivative
  uint8_t* satcheck;     // fluid-soil: Particle::SatCheck of this step
  double* fsi_p;         // fluid-solid: Particle::FSIPressure of this step (0 without FSI)
  double4_32a* fsi_nsv;  // fluid-solid: Particle::FSINSv of this step
  double* sumden;
  double* sumkernel;
  double4_32a* nsv4;     // wall no-slip velocity
  double4_32a* vxsph4;   // XSPH velocity correction
  double* strain_rate;   // 9 per particle
  double* rotation_rate; // 9 per particle
  double* shear_rate;
  double* sbar;
  double* sigma_o;       // leapfrog Sigmab | MVerlet Sigmaa: per-step output only (9 per particle)
  double* strain_o;      // leapfrog Strainb | MVerlet Straina
  double* shear_o;       // leapfrog ShearStressb | MVerlet ShearStressa
  // learned closure (allocated when attached)
  float* cvort;          // |vorticity| from the pair sums
  float* cnnb;           // neighbours inside the support
  float* cshear;         // FP32C: ShearRate of the strain-rate sums
  float* sr32;           // FP32C fluid: the strain-rate sums xx, xy, xz, yy, yz, zz (6 per particle)
  float* cr3;            // FP32C: det(StrainRate) / (StrainRate:StrainRate)^(3/2)
  float* cfeat;          // raw network features, 6 per particle
  double* nut;           // eddy viscosity from the network; -1 = use Smagorinsky
};

struct Options {
  int dim, kt, vis_eq, grad_type, scheme, wallp_physical;
  int fp32;           // PSPH_FP32C pair arithmetic
  int has_solid;      // any Material 2/3
  int any_av;         // any alpha/beta != 0
  int any_ti;         // any TI > 0
  int need_sr;        // strain rate needed (fluid T0>0 or LES)
  int any_shepard;
  int uniform_eos;    // all free particles of the material share one EOS class
  int eos_cls;        // that class
  int dyn_mu;
  int in_out_flow;    // Domain::BC.InOutFlow (single FP64 fluid domain)
  double out_density; // BC.outDensity (whether out-flow particles keep their density)
  int soil_pairs;     // Material 3 (soil-soil walls take the partner's density)
  int mixed;          // fluid (Material 1) and a soil or a solid share the domain: each pair
                      // kernel keeps to its material, a coupling kernel adds the pairs of
                      // different materials (FP64 form)
  int couple_soil;    // fluid + soil: CalcForce13, the saturation switch
  int couple_solid;   // fluid + solid: CalcForce12
  int fsi;            // Domain::FSI: the solid's interpolated pressure and velocity
  int swi;            // Domain::SWIType
  int carry_shear_h;  // the sort moves the ShearStress history (Mat2, or a non-zero upload)
  int uniform_h;      // every particle has the same h
  int any_periodic;   // some instance has a periodic axis
  int any_periodic_x; // some instance has a periodic x axis (no staged neighbour scan)
  int fp64_half;      // FP64 fluid pair forces evaluate each pair once (no strain rate, XSPH or solids)
  int uniform_mu;     // every free particle has the same constant viscosity
  int uniform_av;     // every class has the same artificial-viscosity alpha and beta (alpha32, beta32)
  int uniform_mass;   // every free class has one mass (m_free32), every fixed class one FPMassC (fpm_wall32)
  float alpha32, beta32, m_free32, fpm_wall32;
  double mu_u;        // that viscosity
  double inv_h;       // 1/h when uniform
  int nl_cap;         // neighbour-list capacity per particle
  int pair_block;     // threads per block of the FP32C pair kernels (psph_autotune)
  int xsub;           // x-slabs per cell in the sort (1, 2 or 4; psph_autotune)
  int nlist_stage;    // staged candidates per block of the neighbour scan (0 = global; psph_autotune)
  double xsph, sqrt_h_a;
  double gravity[3], body_force[3];
  double gb[3];       // gravity + body force (the sum every pair kernel starts from)
  float skin;         // FP32C neighbour lists with a skin (fraction of the support); 0: rebuilt every step
  float skin_disp2;   // the smallest of the instances' GridDev::skin_disp2
  int a_from_hook;    // FP64 pair kernels start from this step's A4 (set by a GeneralBefore
                      // hook, Source/Domain.cpp:1767) instead of Gravity
  // FP32 copies for the FP32C kernels, converted once on the host (a
  // double-to-float conversion on the device runs on the FP64 pipe)
  float inv_h32, mu_u32, xsph32, sqrt_h_a32, gravity32[3];
  int shepard_step;
  int nclasses;
  int closure;        // learned eddy-viscosity closure attached
  double closure_dx;  // lattice spacing of its h/dx feature
};

// Chunk stride of the neighbour lists (nl_slot permutes particles inside
// blocks of 64): the capacity rounded up to a multiple of 64.
inline int nl_stride_of(int ncap) { return (ncap + 63) & ~63; }

// Everything a launch needs, passed by value to the launch wrappers.
struct DevView {
  const GridDev* grids;   // per instance (device array): the cells of the sort and the lists
  const GridDev* grids_ref;  // the reference's grids (CellInitiate); the same as grids without a skin
  InstState* inst;        // per instance
  int ninst;
  int total_cells;        // sum of the instances' cells
  Options o;
  Persist PA, PB; // double-buffered persistent arrays; StepScalars::buf says which is current
  Scratch S;
  const PClass* cls;
  const PClass32* cls32;
  const void* mlp;        // closure network image (MlpImage), when attached
  StepScalars* sc;
  uint8_t* alive;
  int ncap;
  int nl_stride;          // neighbour-list chunk stride: ncap rounded up to a multiple of 64 (nl_slot)
  int nclasses;
};

PSPH_D const GridDev& grid_of(const DevView& v, int inst) { return v.grids[inst]; }

PSPH_D const Persist& cur_persist(const DevView& v) { return v.sc->buf ? v.PB : v.PA; }
PSPH_D const Persist& next_persist(const DevView& v) { return v.sc->buf ? v.PA : v.PB; }

// Launch wrappers (defined in the .cu files).
void launch_sort(const DevView& v, cudaStream_t st);      // bin + scan + scatter + rank + reorder + flip
void launch_nlist(const DevView& v, cudaStream_t st);     // per-step neighbour lists
void launch_skin_offsets(const DevView& v, cudaStream_t st);  // lists with a skin: FP32 offsets, reference cells
// the next cell sort runs (now, a sort outside a step) / the next step rebuilds its lists
void launch_mark_rebuild(const DevView& v, bool now, bool next_step, cudaStream_t st);
void nlist_configure();                                   // once, outside stream capture: shared-memory limits
void launch_prepare(const DevView& v, cudaStream_t st);   // per-particle derived quantities, TIR
void launch_prepare32(const DevView& v, cudaStream_t st); // FP32C form: copies + wall interpolation
void launch_forces32(const DevView& v, cudaStream_t st);  // FP32C form: fluid pair forces
void launch_expand_sr32(const DevView& v, int n, cudaStream_t st);  // sr32 -> the FP64 strain_rate tensors
void launch_wall(const DevView& v, cudaStream_t st);      // wall interpolation
void launch_forces(const DevView& v, cudaStream_t st);    // pair forces + per-block dt minimum
void launch_saturation(const DevView& v, cudaStream_t st); // fluid-soil: saturation check and weight switch
void launch_fsi(const DevView& v, cudaStream_t st);       // fluid-solid: FSI interpolation of the solid
void launch_coupling(const DevView& v, cudaStream_t st);  // pairs of different materials (CalcForce12/13) + dt
void launch_dt(const DevView& v, cudaStream_t st);        // dt reduction + AdaptiveTimeStep
void launch_update(const DevView& v, cudaStream_t st);    // Move + material update + periodic wrap + leave
void launch_begin(const DevView& v, cudaStream_t st);     // stop test, first-step counters
void launch_end(const DevView& v, cudaStream_t st);       // time, counters
void launch_closure(const DevView& v, cudaStream_t st);   // learned eddy viscosity (tcgen05 MLP)
int forces_blocks(int ncap);
void launch_class_constants(PClass* cls, int n, int dim, cudaStream_t st);  // derived class constants, once per upload
int launches_per_step(const DevView& v);
void launch_pairs_export(const DevView& v, int which, long long* out, long long cap, unsigned long long* counter,
                         cudaStream_t st);

}  // namespace psph

namespace psph {
// Pieces of the two-pass pair export (scratch supplied by the caller).
void launch_exclusive_scan(const int* in, int* out, int len, int* block_sums, cudaStream_t st);
// upload: the caller's arrays, copied to the device as they are, into the persistent layout
void launch_upload_pack(const double* sx, const double* sd, const double* sp, const double* sv, const double* sh1,
                        const double* sh1s, const double* sh2, const double* sh2s, const double* smu, const Persist& P,
                        int n, bool two_d, bool lf, bool dyn_mu, cudaStream_t st);
void launch_pairs_count(const DevView& v, int which, int* counts, cudaStream_t st);
void launch_pairs_write(const DevView& v, int which, const int* offsets, long long* out, long long cap,
                        cudaStream_t st);
}  // namespace psph
