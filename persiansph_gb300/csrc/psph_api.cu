// C ABI of the GB300 hot path (include/psph.h): context, upload/download,
// Solve's set-up on the host (InitialChecks, CellInitiate, TimestepCheck), and
// the per-step launch sequence captured once into a CUDA graph.
//
// A context holds one or more independent instances (domains). A single
// SPH::Domain is a one-instance context; an ensemble (psph_batch_*) puts all
// instances in the same device arrays: each instance keeps its own cell grid
// (a block of global cell ids), its own time step and stop time, and the same
// kernel launches serve all of them, so a step is one graph launch whatever
// the number of instances.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <unistd.h>
#include <unordered_map>
#include <mutex>
#include <vector>

#include "psph_device.cuh"
#include "psph_inout.cuh"
#include "psph_mlp.cuh"
#include "psph_output.cuh"

using namespace psph;

// Phases timed by psph_phase_times: sort, neighbour lists, prepare, pair
// forces, closure, dt, update.
constexpr int kNumPhases = 7;
// Finest split of the cells into x-slabs in the sort (Options::xsub).
constexpr int kMaxXsub = 4;
// Deepest staging of the neighbour search (Options::nlist_stage, candidates per block).
constexpr int kMaxStage = 4096;
constexpr int kMaxSkinPermille = 150;  // list skins up to 15 % of the support (the lists' capacity)

struct psph_ctx {
  int ninst = 1;
  std::vector<psph_config> cfgs;
  std::vector<psph_grid> grids;  // Domain::CellNo/CellSize/BLPF/TRPR/hmax per instance
  std::vector<psph_integrator> integ;
  bool grid_set = false;  // single-domain continuation (psph_set_grid)
  bool integ_set = false;
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int ncap = 0;
  std::vector<int64_t> inst_off;  // original-index range [inst_off[q], inst_off[q+1]) of instance q
  // download scratch (allocated at the first download): output row of each
  // sorted particle, its scan, and a staging buffer in the caller's layout
  int *dl_flag = nullptr, *dl_rank = nullptr, *dl_row = nullptr, *dl_bs = nullptr;
  size_t dl_cap = 0;  // entries of dl_flag / dl_rank
  double* dl_buf = nullptr;
  int dl_width = 0;
  std::vector<PClass> classes;
  Options opt{};
  std::vector<GridDev> gdevs;
  int total_cells = 0;
  Persist PA{}, PB{};
  Scratch S{};
  PClass* d_cls = nullptr;
  PClass32* d_cls32 = nullptr;
  GridDev* d_grids = nullptr;           // the lists' and the sort's grids (the reference's without a skin)
  GridDev* d_grids_ref = nullptr;       // the reference's grids (CellInitiate)
  int total_cells_ref = 0;
  InstState* d_inst = nullptr;
  InstState* h_inst = nullptr;  // pinned mirror
  StepScalars* d_sc = nullptr;
  StepScalars* h_sc = nullptr;  // pinned mirror
  uint8_t* d_alive = nullptr;
  MlpImage* d_mlp = nullptr;  // closure network (copied at psph_closure_attach)
  std::vector<void*> allocs;
  cudaGraphExec_t graph = nullptr;
  bool uploaded = false;
  bool timing = false;
  double phase_ms[kNumPhases] = {};
  double tuned_ms = 0.0;  // psph_autotune's measured time per step
  long long last_launches = 0;
  // snapshot output (psph_output_request / psph_output_write)
  OutputWriter* out = nullptr;
  bool out_requested = false;
  std::string out_key, out_names[3];
  cudaEvent_t ev[kNumPhases + 1] = {};
  // in/out-flow boundary (one FP64 fluid domain): BC state and the
  // reference's ordered lists, kept on the host (psph_inout.cu holds the kernels)
  bool inout = false;
  int inoutcounter = 0;                 // BC.inoutcounter
  double in_loc1 = 0.0, in_loc2 = 0.0, in_loc3 = 0.0, out_loc = 0.0;
  std::vector<long long> in_part;       // BC.InPart (original indices), in list order
  long long next_orig = 0;              // original index of the next appended particle
  int* d_slot_of = nullptr;             // slot of each original index
  long long slot_cap = 0;
  int* d_flow_count = nullptr;
  void* d_flow_buf = nullptr;           // candidates / slots / recycle commands
  size_t flow_buf_bytes = 0;
  int cls_cap = 0;                      // device class-table capacity
  psph_flow_fn flow_fn[3] = {};         // user InCon / OutCon (PSPH_FLOW_IN / PSPH_FLOW_OUT); null: the constants
  void* flow_user[3] = {};
  // host hooks inside a step (GeneralBefore / GeneralAfter, psph_set_step_hooks)
  psph_hook_fn hook_fn = nullptr;
  void* hook_user = nullptr;
  int hook_mask = 0;
  int in_hook = 0;                      // PSPH_HOOK_* while a hook runs
  bool hook_set_a = false;              // the GeneralBefore hook patched accelerations or density rates
  bool hook_set_x = false;              // ... or positions (the FP32 cell offsets follow)
  std::map<std::string, int> class_index;  // class record -> index (classes added as particles are recycled)
};

namespace {

psph_status set_err(psph_ctx* c, psph_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CUDA_TRY(ctx, call)                                                                      \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return set_err(ctx, e_ == cudaErrorMemoryAllocation ? PSPH_ERR_OUT_OF_MEMORY : PSPH_ERR_CUDA, \
                     "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);        \
  } while (0)

template <class T>
psph_status dalloc(psph_ctx* c, T** p, size_t count) {
  void* ptr = nullptr;
  if (count == 0) count = 1;
  CUDA_TRY(c, cudaMalloc(&ptr, count * sizeof(T)));
  CUDA_TRY(c, cudaMemset(ptr, 0, count * sizeof(T)));
  c->allocs.push_back(ptr);
  *p = (T*)ptr;
  return PSPH_OK;
}

void free_all(psph_ctx* c) {
  if (c->graph) cudaGraphExecDestroy(c->graph);
  c->graph = nullptr;
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
  if (c->h_sc) cudaFreeHost(c->h_sc);
  c->h_sc = nullptr;
  if (c->h_inst) cudaFreeHost(c->h_inst);
  c->h_inst = nullptr;
}

// Particle constructor defaults (Source/Particle.cpp:25-117) for NULL arrays.
double dflt(const double* a, int64_t i, double d) { return a ? a[i] : d; }
int32_t iflt(const int32_t* a, int64_t i, int32_t d) { return a ? a[i] : d; }


// Threads for the per-particle host loops of an upload (one per ~200k
// particles, at most the hardware's).
int host_threads(int64_t n) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  return (int)std::max<int64_t>(1, std::min<int64_t>(hw, n / 200000 + 1));
}

template <class F>
void run_threads(int n, F&& f) {
  if (n <= 1) {
    f(0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < n; ++t) th.emplace_back(f, t);
  f(0);
  for (auto& x : th) x.join();
}

// CellInitiate (Source/Domain.cpp:549-660) for one instance.
psph_status cell_initiate(psph_ctx* c, const psph_config& cf, const psph_particles* p, psph_grid& g,
                          double* mu_max, double* cs_max) {
  const int64_t n = p->n;
  // extremes over the particles, per thread chunk then merged (the same
  // comparisons, so the result does not depend on the split)
  struct Ext {
    double TRPR[3], BLPF[3], hmax, rhomax, mu_max, cs_max;
  };
  const int nth = host_threads(n);
  std::vector<Ext> part(nth);
  run_threads(nth, [&](int t) {
    Ext& E = part[t];
    for (int d = 0; d < 3; ++d) E.TRPR[d] = E.BLPF[d] = p->x[d];
    E.hmax = p->h[0];
    E.rhomax = p->density[0];
    E.mu_max = E.cs_max = 0.0;
    for (int64_t i = n * t / nth; i < n * (t + 1) / nth; ++i) {
      for (int d = 0; d < 3; ++d) {
        const double xd = p->x[3 * i + d];
        if (xd > E.TRPR[d]) E.TRPR[d] = xd;
        if (xd < E.BLPF[d]) E.BLPF[d] = xd;
      }
      if (p->h[i] > E.hmax) E.hmax = p->h[i];
      if (p->density[i] > E.rhomax) E.rhomax = p->density[i];
      const double mu = dflt(p->mu, i, 0.0), cs = dflt(p->cs, i, 0.0);
      if (mu > E.mu_max) E.mu_max = mu;
      if (cs > E.cs_max) E.cs_max = cs;
    }
  });
  double TRPR[3], BLPF[3];
  for (int d = 0; d < 3; ++d) TRPR[d] = BLPF[d] = p->x[d];
  double hmax = p->h[0];
  double rhomax = p->density[0];
  *mu_max = 0.0;
  *cs_max = 0.0;
  for (const Ext& E : part) {
    for (int d = 0; d < 3; ++d) {
      if (E.TRPR[d] > TRPR[d]) TRPR[d] = E.TRPR[d];
      if (E.BLPF[d] < BLPF[d]) BLPF[d] = E.BLPF[d];
    }
    if (E.hmax > hmax) hmax = E.hmax;
    if (E.rhomax > rhomax) rhomax = E.rhomax;
    if (E.mu_max > *mu_max) *mu_max = E.mu_max;
    if (E.cs_max > *cs_max) *cs_max = E.cs_max;
  }
  for (int d = 0; d < 3; ++d) {
    if (cf.dom_max[d] > TRPR[d]) TRPR[d] = cf.dom_max[d];
    if (cf.dom_min[d] < BLPF[d]) BLPF[d] = cf.dom_min[d];
  }
  for (int d = 0; d < 3; ++d) {
    if (!cf.periodic[d]) {
      TRPR[d] += hmax / 2;
      BLPF[d] -= hmax / 2;
    } else {
      TRPR[d] += cf.R;
      BLPF[d] -= cf.R;
    }
  }
  const double cellfac = (cf.kernel_type == PSPH_QUINTIC_SPLINE) ? 3.0 : 2.0;
  for (int d = 0; d < 3; ++d) {
    if (d < cf.dimension) {
      const double r = (TRPR[d] - BLPF[d]) / (cellfac * hmax);
      if ((double)(std::ceil(((TRPR[d] - BLPF[d]) / (cellfac * hmax))) - r) < (hmax / 10.0)) g.cell_no[d] = (int)std::ceil(r);
      else g.cell_no[d] = (int)std::floor(r);
      if (g.cell_no[d] < 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "domain thinner than one cell on axis %d", d);
      g.cell_size[d] = (TRPR[d] - BLPF[d]) / g.cell_no[d];
    } else {
      g.cell_no[d] = 1;
      g.cell_size[d] = 0.0;
    }
  }
  for (int d = 0; d < 3; ++d) {
    if (cf.periodic[d]) g.cell_no[d] += 2;
    g.dom_size[d] = cf.periodic[d] ? (TRPR[d] - BLPF[d]) : 0.0;
    g.blpf[d] = BLPF[d];
    g.trpr[d] = TRPR[d];
  }
  g.hmax = hmax;
  g.rhomax = rhomax;
  g.cellfac = cellfac;
  return PSPH_OK;
}

struct ClassKeyHash {
  size_t operator()(const std::string& s) const { return std::hash<std::string>()(s); }
};

void record_phase(psph_ctx* c, int k) {
  if (c->timing) cudaEventRecord(c->ev[k], c->stream);
}

DevView view(psph_ctx* c) {
  DevView v{};
  v.grids = c->d_grids;
  v.grids_ref = c->d_grids_ref;
  v.inst = c->d_inst;
  v.ninst = c->ninst;
  v.total_cells = c->total_cells;
  v.o = c->opt;
  v.PA = c->PA;
  v.PB = c->PB;
  v.S = c->S;
  v.cls = c->d_cls;
  v.cls32 = c->d_cls32;
  v.mlp = c->d_mlp;
  v.sc = c->d_sc;
  v.alive = c->d_alive;
  v.ncap = c->ncap;
  v.nl_stride = nl_stride_of(c->ncap);
  v.nclasses = (int)c->classes.size();
  return v;
}

// The view on the reference's cell grid (the same as view() without a skin):
// the pair exports list the reference's candidate pairs in its orientation.
DevView view_ref(psph_ctx* c) {
  DevView v = view(c);
  v.grids = c->d_grids_ref;
  v.total_cells = c->total_cells_ref;
  return v;
}

// One step of Solve's loop body (Source/Domain.cpp:1764-1792) as launches;
// before_update (if given) enqueues work between the forces and the update,
// where Solve writes its output (Source/Domain.cpp:1773-1788).
template <class F>
void enqueue_step(psph_ctx* c, F&& before_update);
void enqueue_step(psph_ctx* c) {
  enqueue_step(c, [] {});
}
template <class F>
void enqueue_step(psph_ctx* c, F&& before_update) {
  const DevView v = view(c);
  cudaStream_t st = c->stream;
  launch_begin(v, st);
  record_phase(c, 0);
  launch_sort(v, st);
  record_phase(c, 1);
  launch_nlist(v, st);
  if (v.o.skin > 0.f) launch_skin_offsets(v, st);
  record_phase(c, 2);
  if (v.o.fp32) launch_prepare32(v, st);
  else launch_prepare(v, st);
  if (v.o.couple_soil && v.o.swi != 2) launch_saturation(v, st);
  if (v.o.fsi) launch_fsi(v, st);
  record_phase(c, 3);
  if (v.o.fp32) launch_forces32(v, st);
  else launch_forces(v, st);
  if (v.o.mixed) launch_coupling(v, st);
  record_phase(c, 4);
  if (v.o.closure) launch_closure(v, st);
  record_phase(c, 5);
  launch_dt(v, st);
  before_update();
  record_phase(c, 6);
  launch_update(v, st);
  launch_end(v, st);
  record_phase(c, 7);
}

// Clears every instance's stop flag on the stream, with no stop time (used
// before a pair export, which sorts but does not step). The status word is
// left as the last step set it: an export does not hide a pending error, and
// psph_step clears it when it arms the next run.
__global__ void rearm_kernel(InstState* inst, int ninst, StepScalars* sc) {
  for (int k = threadIdx.x; k < ninst; k += blockDim.x) {
    inst[k].stop = 0;
    inst[k].t_stop = 1e300;
  }
  if (threadIdx.x == 0) sc->all_stop = 0;
}

psph_status sync_scalars(psph_ctx* c) {
  CUDA_TRY(c, cudaMemcpyAsync(c->h_sc, c->d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(c->h_inst, c->d_inst, sizeof(InstState) * c->ninst, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return PSPH_OK;
}

// Sets each instance's stop time (t_stop[q], or t_all when t_stop is NULL)
// and clears the stop flags and the status word before a run of steps.
psph_status arm(psph_ctx* c, const double* t_stop, double t_all) {
  psph_status st = sync_scalars(c);
  if (st) return st;
  for (int q = 0; q < c->ninst; ++q) {
    c->h_inst[q].t_stop = t_stop ? t_stop[q] : t_all;
    c->h_inst[q].stop = 0;
  }
  c->h_sc->status = 0;
  c->h_sc->all_stop = 0;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_inst, c->h_inst, sizeof(InstState) * c->ninst, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(c->d_sc, c->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return PSPH_OK;
}

psph_status build_graph(psph_ctx* c) {
  if (c->graph) return PSPH_OK;
  cudaGraph_t g;
  CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_step(c);
  cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
  if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
  return PSPH_OK;
}

psph_status create_impl(const psph_config* cfgs, int ninst, psph_ctx** out) {
  if (!cfgs || !out || ninst < 1) return PSPH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  psph_ctx* c = new psph_ctx();
  *out = c;
  c->ninst = ninst;
  c->cfgs.assign(cfgs, cfgs + ninst);
  for (int q = 0; q < ninst; ++q) {
    const psph_config& k = cfgs[q];
    if (k.dimension != 2 && k.dimension != 3)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Please correct the dimension (2=>2D or 3=>3D) and run again");
    if (k.kernel_type < 0 || k.kernel_type > 2)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Kernel Type No is out of range");
    if (k.vis_eq < 0 || k.vis_eq > 3) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Viscosity Equation No is out of range");
    if (k.gradient_type < 0 || k.gradient_type > 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Gradient type out of range");
    if (k.scheme != PSPH_MVERLET && k.scheme != PSPH_LEAPFROG)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Scheme must be 0 (Modified Verlet) or 1 (Leapfrog)");
    if (k.swi_type < 0 || k.swi_type > 3)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Soil-Water Interaction Type No is out of range");
    if (k.in_out_flow < 0 || k.in_out_flow > 3) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "InOutFlow is out of range");
    if (k.in_out_flow > 0 && k.periodic[0])
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT,
                     "Periodic BC in the X direction cannot be used with In/Out-Flow BC simultaneously");
    if (k.precision != PSPH_FP64 && k.precision != PSPH_FP32C)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "precision must be PSPH_FP64 or PSPH_FP32C");
    if (k.dimension == 2 && k.periodic[2]) return set_err(c, PSPH_ERR_UNSUPPORTED, "periodic z in 2D");
    for (int e = 0; e < 5; ++e)
      if (k.reserved[e]) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "reserved fields must be zero");
    // one set of kernels serves all instances: the physics switches must agree
    const psph_config& a = cfgs[0];
    bool same = k.dimension == a.dimension && k.kernel_type == a.kernel_type && k.vis_eq == a.vis_eq &&
                k.gradient_type == a.gradient_type && k.scheme == a.scheme && k.precision == a.precision &&
                k.wall_pressure_mode == a.wall_pressure_mode && k.shepard_step == a.shepard_step &&
                k.xsph == a.xsph && k.sqrt_h_a == a.sqrt_h_a && k.swi_type == a.swi_type &&
                k.in_out_flow == a.in_out_flow;
    for (int d = 0; d < 3; ++d) same = same && k.gravity[d] == a.gravity[d] && k.body_force[d] == a.body_force[d];
    if (!same)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT,
                     "instance %d: an ensemble shares dimension, kernel, viscosity, gradient, scheme, precision, "
                     "wall pressure, gravity, body force, XSPH, sqrt_h_a, Shepard step and SWIType with instance 0",
                     q);
  }
  int dev = 0;
  if (psph_device_check(&dev) != PSPH_OK) return set_err(c, PSPH_ERR_NO_DEVICE, "no sm_103 CUDA device available");
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  c->own_stream = true;
  for (int i = 0; i <= kNumPhases; ++i) cudaEventCreate(&c->ev[i]);
  c->grids.resize(ninst);
  c->integ.resize(ninst);
  for (int q = 0; q < ninst; ++q) {
    std::memset(&c->grids[q], 0, sizeof(psph_grid));
    psph_integrator& it = c->integ[q];
    std::memset(&it, 0, sizeof it);
    it.time = cfgs[q].time;
    it.deltat = it.deltatint = it.deltatmin = cfgs[q].dt;
    it.first_step = 1;
  }
  return PSPH_OK;
}


// The options that follow from the parameter sets: which pair terms any
// particle needs and which constants every particle shares (the kernels take
// those from the launch parameters).
void derive_class_options(const std::vector<PClass>& classes, bool mixed, bool dyn_mu, Options& o) {
  o.uniform_eos = 1;
  o.eos_cls = -1;
  o.uniform_h = 1;
  o.any_av = o.any_ti = o.need_sr = o.any_shepard = 0;
  for (size_t q = 0; q < classes.size(); ++q) {
    const PClass& C = classes[q];
    if (C.h != classes[0].h) o.uniform_h = 0;
    if (C.alpha != 0.0 || C.beta != 0.0) o.any_av = 1;
    if (C.ti > 0.0) o.any_ti = 1;
    if (C.material == 1 && (C.t0 > 0.0 || C.les)) o.need_sr = 1;
    if (C.shepard) o.any_shepard = 1;
    if (C.is_free && (!mixed || C.material == 1)) {  // the fluid's EOS (walls take it from the fluid)
      if (o.eos_cls < 0) o.eos_cls = (int)q;
      else {
        const PClass& E = classes[o.eos_cls];
        if (E.pres_eq != C.pres_eq || E.cs != C.cs || E.p0 != C.p0 || E.rho0 != C.rho0) o.uniform_eos = 0;
      }
    }
  }
  if (o.eos_cls < 0) o.eos_cls = 0;
  // two materials: a wall takes its density from its partner's EOS pair by pair
  if (mixed) o.uniform_eos = 0;
  // pair constants that are the same for every class: the FP32C fluid pair
  // loop takes them from the launch parameters (the same FP32 values the class
  // table holds, so the results are identical)
  {
    o.uniform_av = o.uniform_mass = 1;
    const PClass& C0 = classes[0];
    double m_free = -1.0, fpm_wall = -1.0;
    for (const PClass& C : classes) {
      if (C.alpha != C0.alpha || C.beta != C0.beta) o.uniform_av = 0;
      double& ref = C.is_free ? m_free : fpm_wall;
      const double val = C.is_free ? C.mass : C.fpmassc;
      if (ref < 0.0) ref = val;
      else if (val != ref) o.uniform_mass = 0;
    }
    o.alpha32 = (float)C0.alpha;
    o.beta32 = (float)C0.beta;
    o.m_free32 = (float)std::max(m_free, 0.0);
    o.fpm_wall32 = (float)std::max(fpm_wall, 0.0);
  }
  o.uniform_mu = !dyn_mu;
  o.mu_u = 0.0;
  {
    bool first = true;
    for (const PClass& C : classes)
      if (C.is_free) {
        if (first) { o.mu_u = C.mu0; first = false; }
        else if (C.mu0 != o.mu_u) o.uniform_mu = 0;
      }
    // zero viscosity keeps the reference's 0/0 harmonic mean (Source/Interaction.cpp:103)
    if (!(o.mu_u > 0.0)) o.uniform_mu = 0;
  }
  o.inv_h = 1.0 / classes[0].h;
}

psph_status upload_impl(psph_ctx* c, const psph_particles* parts, int initial) {
  if (!c || !parts) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->uploaded) return set_err(c, PSPH_ERR_STATE, "particles already uploaded to this context");
  if (!c->stream) return set_err(c, PSPH_ERR_STATE, "context not created");
  nlist_configure();  // shared-memory limit of the staged neighbour scan (outside any capture)
  const int ninst = c->ninst;
  const psph_config& k = c->cfgs[0];
  const bool lf = (k.scheme == PSPH_LEAPFROG);
  int64_t ntot = 0;
  c->inst_off.assign(ninst + 1, 0);
  for (int q = 0; q < ninst; ++q) {
    const psph_particles* p = &parts[q];
    if (p->n < 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, ninst == 1 ? "no particles" : "instance %d has no particles", q);
    if (p->n > (1LL << 30)) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "too many particles");
    if (!p->x || !p->h || !p->density || !p->mass)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "x, h, density and mass are required (instance %d)", q);
    c->inst_off[q] = ntot;
    ntot += p->n;
  }
  c->inst_off[ninst] = ntot;

  // ---- particle classes (per instance) and initial pressure -------------------
  // Host work over every particle, split across threads: each thread
  // de-duplicates the parameter sets of its contiguous chunk; the chunks'
  // tables merge in chunk order, so class ids do not depend on scheduling.
  bool dyn_mu = false;
  for (int q = 0; q < ninst && !dyn_mu; ++q) {
    const psph_particles& pq = parts[q];
    if (!pq.t0 && !pq.les) continue;
    const int nth = host_threads(pq.n);
    std::vector<char> found(nth, 0);
    run_threads(nth, [&](int t) {
      for (int64_t i = pq.n * t / nth; i < pq.n * (t + 1) / nth; ++i)
        if (dflt(pq.t0, i, 0.0) > 0.0 || iflt(pq.les, i, 0)) {
          found[t] = 1;
          break;
        }
    });
    for (char f : found) dyn_mu = dyn_mu || f;
  }
  // per-particle class and initial pressure, written by the workers below
  // (left uninitialised here: their pages are first touched in parallel)
  std::unique_ptr<int[]> cls_buf(new int[ntot > 0 ? ntot : 1]);
  std::unique_ptr<double[]> pressure_buf(new double[ntot > 0 ? ntot : 1]);
  int* const cls = cls_buf.get();
  double* const pressure = pressure_buf.get();
  struct Worker {
    std::vector<PClass> classes;
    std::unordered_map<std::string, int, ClassKeyHash> index;
    int materials = 0;  // bit m: Material m present
    int64_t err_at = -1;
    psph_status err = PSPH_OK;
    char msg[160] = {0};
  };
  const int nthreads = host_threads(ntot);
  std::vector<Worker> workers(nthreads);
  auto work = [&](int t) {
    Worker& W = workers[t];
    const int64_t g0 = ntot * t / nthreads, g1 = ntot * (t + 1) / nthreads;
    PClass last;
    std::memset(&last, 0, sizeof last);
    int last_id = -1;
    int q = 0;
    while (q + 1 < ninst && g0 >= c->inst_off[q + 1]) ++q;
    for (int64_t g = g0; g < g1; ++g) {
      while (g >= c->inst_off[q + 1]) ++q;  // the instance of particle g
      const psph_particles* p = &parts[q];
      const int64_t i = g - c->inst_off[q];
#define FAIL(code, ...)                                   \
  do {                                                    \
    W.err = code;                                         \
    W.err_at = g;                                         \
    std::snprintf(W.msg, sizeof W.msg, __VA_ARGS__);      \
    return;                                               \
  } while (0)
      PClass C;
      std::memset(&C, 0, sizeof C);
      C.cs = dflt(p->cs, i, 0.0);
      C.p0 = dflt(p->p0, i, 0.0);
      C.rho0 = p->ref_density ? p->ref_density[i] : p->density[i];
      C.fpmassc = dflt(p->fpmassc, i, 1.0);
      C.alpha = dflt(p->alpha, i, 0.0);
      C.beta = dflt(p->beta, i, 0.0);
      C.mu0 = dyn_mu ? 0.0 : dflt(p->mu, i, 0.0);
      C.mu_ref = dflt(p->mu_ref, i, 0.0);
      C.t0 = dflt(p->t0, i, 0.0);
      C.bm = dflt(p->bingham_m, i, 300.0);
      C.csmag = dflt(p->csmag, i, 0.17);
      C.ti = dflt(p->ti, i, 0.0);
      C.tin = dflt(p->tin, i, 4.0);
      C.tid = dflt(p->ti_init_dist, i, 0.0);
      C.g_mod = dflt(p->g_mod, i, 0.0);
      C.k_mod = dflt(p->k_mod, i, 0.0);
      C.sigmay = dflt(p->sigmay, i, 0.0);
      C.coh = dflt(p->cohesion, i, 0.0);
      C.phi = dflt(p->phi, i, 0.0);
      C.psi = dflt(p->psi, i, 0.0);
      C.h = p->h[i];
      C.mass = p->mass[i];
      C.material = iflt(p->material, i, 0);
      C.is_free = iflt(p->is_free, i, 1) != 0;
      C.no_slip = iflt(p->no_slip, i, 0) != 0;
      C.pres_eq = iflt(p->pres_eq, i, 0);
      C.shepard = iflt(p->shepard, i, 0) != 0;
      C.les = iflt(p->les, i, 0) != 0;
      C.vis_m = iflt(p->vis_m, i, 0);
      C.fail = iflt(p->fail, i, 0);
      C.id = iflt(p->id, i, 0);
      C.inst = q;
      if (C.material == 3) {
        C.seep_type = iflt(p->seepage_type, i, 0);
        C.var_por = iflt(p->var_porosity, i, 0) != 0;
        C.is_sat = iflt(p->is_sat, i, 0) != 0;
        C.n0 = dflt(p->n0, i, 0.0);
        C.kp = dflt(p->k, i, 0.0);
        C.kp2 = dflt(p->k2, i, 0.0);
        C.dgrain = dflt(p->d, i, 0.0);
        C.rho_f = dflt(p->rho_f, i, 0.0);
        // Particle::V: the constructor's Mass / RefDensity unless given
        C.vol = p->volume ? p->volume[i] : C.mass / C.rho0;
        if (C.seep_type < 0 || C.seep_type > 3)
          FAIL(PSPH_ERR_INVALID_ARGUMENT, "Seepage Type No is out of range (particle %lld)", (long long)i);
        // InitialChecks: permeabilities from the porosity (Source/Domain.cpp:1680-1716)
        if (initial) permeability(C.seep_type, C.n0, C.dgrain, &C.kp, &C.kp2);
        // after the first step a free VarPorosity particle's permeabilities follow
        // its strain (the pair kernel derives them): the uploaded values would only
        // split the class table
        if (!initial && C.var_por && C.is_free && C.seep_type >= 1) {
          C.kp = 0.0;
          if (C.seep_type >= 2) C.kp2 = 0.0;
        }
      }
      if (C.material < 1 || C.material > 3)
        FAIL(PSPH_ERR_INVALID_ARGUMENT, "Material Type No is out of range (particle %lld)", (long long)i);
      if (C.pres_eq < 0 || C.pres_eq > 2)
        FAIL(PSPH_ERR_INVALID_ARGUMENT, "Please correct Pressure Equation No (particle %lld)", (long long)i);
      if (C.material == 2 && C.fail > 1) FAIL(PSPH_ERR_INVALID_ARGUMENT, "Undefined failure criteria for solids");
      if (C.material == 3 && C.fail > 3) FAIL(PSPH_ERR_INVALID_ARGUMENT, "Failure Type No is out of range");
      if (C.material == 1 && C.t0 > 0.0 && C.vis_m > 1)
        FAIL(PSPH_ERR_INVALID_ARGUMENT, "Non-Newtonian Viscosity Type No is out of range");
      W.materials |= 1 << C.material;
#undef FAIL
      int id;
      // consecutive particles mostly share their parameters: compare with the
      // previous particle's before building and hashing the key
      if (last_id >= 0 && std::memcmp(&C, &last, sizeof C) == 0) {
        id = last_id;
      } else {
        std::string key((const char*)&C, sizeof C);
        auto it = W.index.find(key);
        if (it == W.index.end()) {
          id = (int)W.classes.size();
          W.index.emplace(key, id);
          W.classes.push_back(C);
        } else {
          id = it->second;
        }
        last_id = id;
        last = C;
      }
      cls[g] = id;  // local to the chunk until the merge below
      // InitialChecks: initial pressure from the EOS for fluids and solids (Source/Domain.cpp:1675-1677)
      const double p_in = dflt(p->pressure, i, 0.0);
      // (the EOS the update applies every step: the Tait power as products, no pow call)
      pressure[g] = (initial && C.material < 3) ? eos(C.pres_eq, C.cs, C.p0, p->density[i], C.rho0) : p_in;
    }
  };
  run_threads(nthreads, work);
  int materials = 0;
  std::unordered_map<std::string, int, ClassKeyHash> index;
  {
    std::vector<std::vector<int>> remaps(nthreads);
    for (int t = 0; t < nthreads; ++t) {
      const Worker& W = workers[t];
      if (W.err) return set_err(c, W.err, "%s", W.msg);
      materials |= W.materials;
      std::vector<int>& remap = remaps[t];
      remap.resize(W.classes.size());
      for (size_t k = 0; k < W.classes.size(); ++k) {
        std::string key((const char*)&W.classes[k], sizeof(PClass));
        auto it = index.find(key);
        if (it == index.end()) {
          const int id = (int)c->classes.size();
          if (id >= 65535) return set_err(c, PSPH_ERR_UNSUPPORTED, "more than 65535 distinct particle parameter sets");
          index.emplace(key, id);
          c->classes.push_back(W.classes[k]);
          remap[k] = id;
        } else {
          remap[k] = it->second;
        }
      }
    }
    // each chunk's local class ids to the merged table's, chunks in parallel
    run_threads(nthreads, [&](int t) {
      const std::vector<int>& remap = remaps[t];
      const int64_t g0 = ntot * t / nthreads, g1 = ntot * (t + 1) / nthreads;
      for (int64_t g = g0; g < g1; ++g) cls[g] = remap[cls[g]];
    });
  }
  // Materials that share a domain: fluid with soil couples through
  // CalcForce13, fluid with a solid through CalcForce12; a solid with a soil
  // has no pair force in the reference (LastComputeAcceleration aborts on it)
  const bool fluid_soil = materials == ((1 << 1) | (1 << 3));
  const bool fluid_solid = materials == ((1 << 1) | (1 << 2));
  const bool mixed = fluid_soil || fluid_solid;
  if (!mixed && (materials & (materials - 1)))
    return set_err(c, PSPH_ERR_UNSUPPORTED,
                   "solid (Material 2) and soil (Material 3) particles share the domain: the reference has no pair "
                   "force for them");
  if (mixed && k.precision != PSPH_FP64)
    return set_err(c, PSPH_ERR_UNSUPPORTED, "domains of two materials run in the FP64 form (PSPH_FP64)");
  const bool inout = k.in_out_flow > 0;
  if (inout) {
    if (ninst != 1) return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow boundaries in an ensemble");
    if (k.precision != PSPH_FP64)
      return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow boundaries run in the FP64 form (PSPH_FP64)");
    if (materials != (1 << 1))
      return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow boundaries with soil or solid particles");
    if (k.periodic[1] || k.periodic[2])
      return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow boundaries with a periodic y or z axis");
    for (const PClass& C : c->classes)
      if (C.shepard)
        return set_err(c, PSPH_ERR_UNSUPPORTED,
                       "Shepard filtering with in/out-flow boundaries (the reference restarts a released "
                       "particle's own Shepard counter)");
  }
  if (fluid_soil) {
    for (int q = 0; q < ninst; ++q)
      if (c->cfgs[q].periodic[1])
        return set_err(c, PSPH_ERR_UNSUPPORTED, "fluid-soil domains with a periodic y axis");
    // Saturation switch (Source/Domain.cpp:1209-1234): a soil particle moves to
    // the class with Mass = V (RefDensity -+ RhoF) and RefDensity -+ RhoF. Each
    // soil class gets that twin; a chain of twins is closed after a few links
    // (later flips return to the previous class, which differs from the
    // reference's repeated -+ RhoF by rounding of RefDensity only).
    if (k.swi_type != 2) {
      std::vector<int> depth(c->classes.size(), 0);
      for (size_t q = 0; q < c->classes.size(); ++q) {
        if (c->classes[q].material != 3) continue;
        const PClass C = c->classes[q];
        PClass T = C;
        T.twin = 0;
        T.mass = C.vol * (C.is_sat ? C.rho0 + C.rho_f : C.rho0 - C.rho_f);
        T.rho0 = C.is_sat ? C.rho0 + C.rho_f : C.rho0 - C.rho_f;
        T.is_sat = !C.is_sat;
        std::string key((const char*)&T, sizeof(PClass));
        auto it = index.find(key);
        int id;
        if (it != index.end()) {
          id = it->second;
        } else if (depth[q] >= 3) {
          id = -1;  // closed below
        } else {
          id = (int)c->classes.size();
          if (id >= 65535) return set_err(c, PSPH_ERR_UNSUPPORTED, "more than 65535 distinct particle parameter sets");
          index.emplace(key, id);
          c->classes.push_back(T);
          depth.push_back(depth[q] + 1);
        }
        c->classes[q].twin = id;
      }
      for (size_t q = 0; q < c->classes.size(); ++q)
        if (c->classes[q].material == 3 && c->classes[q].twin < 0)
          for (size_t r = 0; r < c->classes.size(); ++r)
            if (c->classes[r].twin == (int)q) c->classes[q].twin = (int)r;  // back to the class it came from
    }
  }

  // ---- grids (CellInitiate) and TimestepCheck, per instance --------------------
  c->gdevs.resize(ninst);
  long long cell_base = 0;
  for (int q = 0; q < ninst; ++q) {
    const psph_config& cf = c->cfgs[q];
    psph_grid& g = c->grids[q];
    if (!(c->grid_set && q == 0)) {
      double mu_max, cs_max;
      psph_status st = cell_initiate(c, cf, &parts[q], g, &mu_max, &cs_max);
      if (st) return st;
      if (initial) {  // TimestepCheck (Source/Domain.cpp:1721-1733)
        const double t1 = 0.25 * g.hmax / (cs_max);
        const double t2 = (mu_max > 0.0) ? 0.125 * g.hmax * g.hmax * g.rhomax / mu_max : 1000000.0;
        if (c->integ[q].deltatint > std::min(t1, t2))
          return set_err(c, PSPH_ERR_CFL, "Please decrease the time step to the allowable range (CFL limit %g s)",
                         std::min(t1, t2));
      }
    }
    GridDev& gd = c->gdevs[q];
    std::memset(&gd, 0, sizeof gd);
    for (int d = 0; d < 3; ++d) {
      gd.blpf[d] = g.blpf[d];
      gd.trpr[d] = g.trpr[d];
      gd.cell_size[d] = g.cell_size[d];
      gd.dom_size[d] = g.dom_size[d];
      gd.periodic[d] = cf.periodic[d] ? 1 : 0;
      gd.cn_ref[d] = g.cell_no[d];
      gd.nc[d] = cf.periodic[d] ? g.cell_no[d] - 2 : g.cell_no[d];
      if (cf.periodic[d] && gd.nc[d] < 3)
        return set_err(c, PSPH_ERR_UNSUPPORTED, "periodic axis %d spans fewer than 3 cells", d);
    }
    gd.hmax = g.hmax;
    for (int d = 0; d < 3; ++d) gd.inv_cell_size32[d] = (float)(1.0 / g.cell_size[d]);
    for (int d = 0; d < 3; ++d) gd.cell_size32[d] = (float)g.cell_size[d];
    gd.cellfac = (cf.kernel_type == PSPH_QUINTIC_SPLINE) ? 3.0 : 2.0;
    gd.cellfac2_32 = (float)(gd.cellfac * gd.cellfac);
    g.cellfac = gd.cellfac;
    const long long nci = (long long)gd.nc[0] * gd.nc[1] * gd.nc[2];
    if (nci > (1LL << 28)) return set_err(c, PSPH_ERR_UNSUPPORTED, "grid has more than 2^28 cells");
    gd.ncells = (int)nci;
    gd.cell_base = (int)cell_base;
    cell_base += nci;
    if (cell_base > (1LL << 28))
      return set_err(c, PSPH_ERR_UNSUPPORTED, "the instances' grids hold more than 2^28 cells");
  }
  c->total_cells = (int)cell_base;
  c->total_cells_ref = c->total_cells;

  // ---- options ---------------------------------------------------------------
  Options& o = c->opt;
  o.dim = k.dimension;
  o.kt = k.kernel_type;
  o.vis_eq = k.vis_eq;
  o.grad_type = k.gradient_type;
  o.scheme = k.scheme;
  o.wallp_physical = (k.wall_pressure_mode == PSPH_WALLP_PHYSICAL);
  o.has_solid = (materials & ((1 << 2) | (1 << 3))) != 0;
  o.mixed = mixed;
  o.in_out_flow = k.in_out_flow;
  o.out_density = k.out_density;
  o.couple_soil = fluid_soil;
  o.couple_solid = fluid_solid;
  o.fsi = fluid_solid && k.fsi != 0;
  o.swi = k.swi_type;
  o.fp32 = (k.precision == PSPH_FP32C);
  if (ntot >= (1LL << 26)) return set_err(c, PSPH_ERR_UNSUPPORTED, "this build handles fewer than 2^26 particles");
  o.soil_pairs = (materials & (1 << 3)) != 0;
  o.dyn_mu = dyn_mu;
  o.xsph = k.xsph;
  o.sqrt_h_a = k.sqrt_h_a;
  o.shepard_step = k.shepard_step;
  for (int d = 0; d < 3; ++d) {
    o.gravity[d] = k.gravity[d];
    o.body_force[d] = k.body_force[d];
  }
  o.uniform_eos = 1;
  o.eos_cls = -1;
  o.uniform_h = 1;
  o.any_periodic = 0;
  o.any_periodic_x = 0;
  for (const GridDev& gd : c->gdevs) {
    if (gd.periodic[0] || gd.periodic[1] || gd.periodic[2]) o.any_periodic = 1;
    if (gd.periodic[0]) o.any_periodic_x = 1;
  }
  derive_class_options(c->classes, mixed, dyn_mu, o);
  for (int d = 0; d < 3; ++d) {
    o.gb[d] = o.gravity[d] + o.body_force[d];
    o.gravity32[d] = (float)o.gravity[d];
  }
  o.inv_h32 = (float)o.inv_h;
  o.mu_u32 = (float)o.mu_u;
  o.xsph32 = (float)o.xsph;
  o.sqrt_h_a32 = (float)o.sqrt_h_a;
  o.nclasses = (int)c->classes.size();
  // neighbour lists: 3D supports hold ~80 (h = 1.3 dx) particles, 2D ~20-44;
  // a particle with more falls back to scanning its cells
  o.nl_cap = (k.dimension == 3) ? 128 : 64;
  // the FP32C form may run its lists with a skin (psph_set_tuning): room for
  // (1 + skin)^3 more entries
  if (k.precision == PSPH_FP32C) o.nl_cap = (k.dimension == 3) ? 160 : 96;
  o.pair_block = 128;
  o.xsub = 1;
  o.nlist_stage = 0;  // measured: the L1-cached scan beats the staged one (psph_autotune tries both)

  // ---- device buffers ----------------------------------------------------------
  // in/out-flow domains gain particles as the in-flow is recycled: headroom
  const int64_t ncap = ntot + (inout ? std::max<int64_t>(1024, ntot / 4) : 0);
  if (ncap >= (1LL << 26)) return set_err(c, PSPH_ERR_UNSUPPORTED, "this build handles fewer than 2^26 particles");
  c->ncap = (int)ncap;
  const size_t N = (size_t)ncap;  // every per-particle array holds the headroom
  psph_status st = PSPH_OK;
  for (Persist* P : {&c->PA, &c->PB}) {
    if ((st = dalloc(c, &P->X4, N)) || (st = dalloc(c, &P->V4, N)) || (st = dalloc(c, &P->H4, N)) ||
        (st = dalloc(c, &P->cls, N)) || (st = dalloc(c, &P->orig, N)))
      return st;
    if (lf && (st = dalloc(c, &P->H4b, N))) return st;
    if (dyn_mu && (st = dalloc(c, &P->mu, N))) return st;
    if (inout && (st = dalloc(c, &P->io, N))) return st;
    if (o.has_solid) {
      if ((st = dalloc(c, &P->sigma, 9 * N)) || (st = dalloc(c, &P->sigma_h, 9 * N)) ||
          (st = dalloc(c, &P->strain, 9 * N)) || (st = dalloc(c, &P->strain_h, 9 * N)) ||
          (st = dalloc(c, &P->shear, 9 * N)) || (st = dalloc(c, &P->shear_h, 9 * N)) ||
          (st = dalloc(c, &P->tir, 9 * N)))
        return st;
    }
  }
  Scratch& S = c->S;
  const size_t NC = (size_t)c->total_cells;
  const size_t NB = NC * kMaxXsub;  // sort bins at the finest x-slab split
  if ((st = dalloc(c, &S.key, N)) || (st = dalloc(c, &S.count, NB + 2)) || (st = dalloc(c, &S.start, NC + 3)) ||
      (st = dalloc(c, &S.sstart, NB + 3)) ||
      (st = dalloc(c, &S.tmp_perm, N)) || (st = dalloc(c, &S.perm, N)) || (st = dalloc(c, &S.cellid, N)) ||
      (st = dalloc(c, &S.block_sums, (NB + 2 + 1023) / 1024 + 1)) ||
      (st = dalloc(c, &S.OFF32, N)) || (st = dalloc(c, &S.D4, N)) || (st = dalloc(c, &S.nl_count, N)) ||
      (st = dalloc(c, &S.A4, N)) || (st = dalloc(c, &S.zwab, N)) || (st = dalloc(c, &S.sumden, N)) ||
      (st = dalloc(c, &S.sumkernel, N)) || (st = dalloc(c, &S.nsv4, N)) || (st = dalloc(c, &S.vxsph4, N)) ||
      (st = dalloc(c, &S.shear_rate, N)) || (st = dalloc(c, &S.sbar, N)))
    return st;
  if (o.couple_soil && o.swi == 1 && (st = dalloc(c, &S.s_acc, N))) return st;
  if (o.couple_soil && o.swi != 2 && (st = dalloc(c, &S.satcheck, N))) return st;
  if (o.couple_solid && ((st = dalloc(c, &S.fsi_p, N)) || (st = dalloc(c, &S.fsi_nsv, N)))) return st;
  if ((st = dalloc(c, &S.nl, (size_t)o.nl_cap * nl_stride_of(c->ncap)))) return st;
  // FP64 fluids without strain-rate sums, XSPH or solids: each pair evaluated once
  o.fp64_half = !o.fp32 && !o.has_solid && !o.need_sr && o.xsph == 0.0;
  if (o.fp64_half) {
    const size_t slots = (size_t)o.nl_cap * nl_stride_of(c->ncap);
    if ((st = dalloc(c, &S.half4, slots)) || (st = dalloc(c, &S.half2, slots)) ||
        (st = dalloc(c, &S.half_stamp, slots)))
      return st;
  }
  if (o.need_sr || o.has_solid)
    if ((st = dalloc(c, &S.strain_rate, 9 * N))) return st;
  if (o.fp32 && ((st = dalloc(c, &S.OFFREF, N)) || (st = dalloc(c, &S.refcell, N)))) return st;
  if (o.fp32) {
    if ((st = dalloc(c, &S.V32, N)) || (st = dalloc(c, &S.D32, N)) || (st = dalloc(c, &S.NSV32, N)) ||
        (st = dalloc(c, &S.V32LO, N)))
      return st;
    if (dyn_mu && (st = dalloc(c, &S.MU32, N))) return st;
    if (o.need_sr && !o.has_solid &&  // FP32 ShearRate and strain-rate sums of the fluid kernel
        ((st = dalloc(c, &S.cshear, N)) || (st = dalloc(c, &S.sr32, 6 * N))))
      return st;
  }
  if (o.fp32 && o.has_solid) {
    if ((st = dalloc(c, &S.SIG32, 2 * N)) || (st = dalloc(c, &S.VB32, N))) return st;
    if (o.any_ti && (st = dalloc(c, &S.TIR32, 2 * N))) return st;
  }
  if (o.has_solid) {
    if ((st = dalloc(c, &S.rotation_rate, 9 * N)) || (st = dalloc(c, &S.sigma_o, 9 * N)) ||
        (st = dalloc(c, &S.strain_o, 9 * N)) || (st = dalloc(c, &S.shear_o, 9 * N)))
      return st;
  }
  c->cls_cap = (int)c->classes.size() + (inout ? 256 : 0);  // recycled in-flow particles may need new classes
  if ((st = dalloc(c, &c->d_cls, (size_t)c->cls_cap)) || (st = dalloc(c, &c->d_sc, 1)) ||
      (st = dalloc(c, &c->d_alive, N)) || (st = dalloc(c, &c->d_grids, (size_t)ninst)) ||
      (st = dalloc(c, &c->d_grids_ref, (size_t)ninst)) ||
      (st = dalloc(c, &c->d_inst, (size_t)ninst)))
    return st;
  CUDA_TRY(c, cudaMallocHost(&c->h_sc, sizeof(StepScalars)));
  CUDA_TRY(c, cudaMallocHost(&c->h_inst, sizeof(InstState) * ninst));
  {
    std::vector<PClass32> c32(c->classes.size());
    for (size_t q = 0; q < c->classes.size(); ++q) {
      const PClass& C = c->classes[q];
      PClass32& F = c32[q];
      F.mass = (float)C.mass; F.h = (float)C.h; F.fpmassc = (float)C.fpmassc; F.alpha = (float)C.alpha;
      F.beta = (float)C.beta; F.mu0 = (float)C.mu0; F.ti = (float)C.ti; F.tin = (float)C.tin; F.tid = (float)C.tid;
      F.cs = (float)C.cs; F.rho0 = (float)C.rho0; F.p0 = (float)C.p0;
      F.flags = (C.is_free ? CF_FREE : 0) | (C.no_slip ? CF_NOSLIP : 0) | (C.les ? CF_LES : 0) |
                (C.shepard ? CF_SHEPARD : 0) | (C.t0 > 0.0 ? CF_T0 : 0) | (C.ti > 0.0 ? CF_TI : 0);
      F.material = C.material;
      F.pres_eq = C.pres_eq;
      F.inst = C.inst;
      F.h_over_dx = c->opt.closure ? (float)(C.h / c->opt.closure_dx) : 0.f;
    }
    if ((st = dalloc(c, &c->d_cls32, c32.size()))) return st;
    CUDA_TRY(c, cudaMemcpy(c->d_cls32, c32.data(), c32.size() * sizeof(PClass32), cudaMemcpyHostToDevice));
  }

  // ---- pack and copy --------------------------------------------------------------
  {
    // The caller's arrays go to the device as they are, into the neighbour-list
    // buffer (free until the first step; 17 doubles per particle fit in its
    // >= 256 bytes), and upload_pack_kernel builds the persistent layout.
    const size_t NN = N;
    double* const sx = reinterpret_cast<double*>(c->S.nl);  // x (3N)
    double* const sd = sx + 3 * NN;                         // density
    double* const sp = sd + NN;                             // initial pressure (from the host loop above)
    double* const sv = sp + NN;                             // v (3N)
    double* const sh1 = sv + 3 * NN;                        // the scheme's history: va (Leapfrog) or vb
    double* const sh1s = sh1 + 3 * NN;                      // densitya or densityb
    double* const sh2 = sh1s + NN;                          // Leapfrog vb
    double* const sh2s = sh2 + 3 * NN;                      // Leapfrog densityb
    double* const smu = sh2s + NN;                          // mu
    auto put = [&](double* dst, const double* src, size_t cnt) -> psph_status {
      if (src) CUDA_TRY(c, cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, c->stream));
      else CUDA_TRY(c, cudaMemsetAsync(dst, 0, cnt * sizeof(double), c->stream));  // the constructor's zero
      return PSPH_OK;
    };
    for (int q = 0; q < ninst; ++q) {
      const psph_particles* p = &parts[q];
      const size_t off = (size_t)c->inst_off[q], m = (size_t)p->n;
      if ((st = put(sx + 3 * off, p->x, 3 * m)) || (st = put(sd + off, p->density, m)) ||
          (st = put(sv + 3 * off, p->v, 3 * m)) || (st = put(sh1 + 3 * off, lf ? p->va : p->vb, 3 * m)) ||
          (st = put(sh1s + off, lf ? p->densitya : p->densityb, m)))
        return st;
      if (lf && ((st = put(sh2 + 3 * off, p->vb, 3 * m)) || (st = put(sh2s + off, p->densityb, m)))) return st;
      if (dyn_mu && (st = put(smu + off, p->mu, m))) return st;
    }
    const size_t NP = (size_t)ntot;  // the particles (N holds the in-flow headroom too)
    if ((st = put(sp, pressure, NP))) return st;
    launch_upload_pack(sx, sd, sp, sv, sh1, sh1s, sh2, sh2s, smu, c->PA, (int)NP, k.dimension == 2, lf, dyn_mu,
                       c->stream);
    CUDA_TRY(c, cudaMemcpyAsync(c->PA.cls, cls, NP * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(c->d_alive, 1, NP, c->stream));
    if (inout && parts[0].in_out)
      CUDA_TRY(c, cudaMemcpyAsync(c->PA.io, parts[0].in_out, NP * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (o.has_solid) {
      // Mat3 neither reads nor writes the ShearStress history: a soil domain
      // whose uploaded history is zero does not carry it through the sort
      o.carry_shear_h = 1;
      if (o.soil_pairs) {
        o.carry_shear_h = 0;
        for (int q = 0; q < ninst && !o.carry_shear_h; ++q) {
          const double* hs = lf ? parts[q].shear_stressa : parts[q].shear_stressb;
          if (hs)
            for (size_t e = 0; e < 9 * (size_t)parts[q].n; ++e)
              if (hs[e] != 0.0) {
                o.carry_shear_h = 1;
                break;
              }
        }
      }
      for (int q = 0; q < ninst; ++q) {
        const psph_particles* p = &parts[q];
        const double* srcs[7] = {p->sigma, lf ? p->sigmaa : p->sigmab, p->strain, lf ? p->straina : p->strainb,
                                 p->shear_stress, lf ? p->shear_stressa : p->shear_stressb, p->tir};
        double* dsts[7] = {c->PA.sigma, c->PA.sigma_h, c->PA.strain, c->PA.strain_h,
                           c->PA.shear, c->PA.shear_h, c->PA.tir};
        const size_t off = 9 * (size_t)c->inst_off[q];
        for (int a = 0; a < 7; ++a)
          if (srcs[a])
            CUDA_TRY(c, cudaMemcpy(dsts[a] + off, srcs[a], 9 * (size_t)p->n * sizeof(double), cudaMemcpyHostToDevice));
      }
    }
    CUDA_TRY(c, cudaMemcpy(c->d_cls, c->classes.data(), c->classes.size() * sizeof(PClass), cudaMemcpyHostToDevice));
    launch_class_constants(c->d_cls, (int)c->classes.size(), o.dim, c->stream);
    CUDA_TRY(c, cudaGetLastError());
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    CUDA_TRY(c, cudaMemcpy(c->d_grids, c->gdevs.data(), ninst * sizeof(GridDev), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_grids_ref, c->gdevs.data(), ninst * sizeof(GridDev), cudaMemcpyHostToDevice));
    std::vector<InstState> is(ninst);
    for (int q = 0; q < ninst; ++q) {
      InstState& I = is[q];
      std::memset(&I, 0, sizeof I);
      const psph_integrator& it = c->integ[q];
      I.time = it.time;
      I.deltat = it.deltat;
      I.deltatint = it.deltatint;
      I.deltatmin = it.deltatmin;
      I.steps = it.steps;
      I.first_step = it.first_step;
      I.k_initial = initial ? 1 : 0;
      I.ct = it.ct;
      I.shepard_counter = it.shepard_counter;
      I.t_stop = 1e300;
    }
    CUDA_TRY(c, cudaMemcpy(c->d_inst, is.data(), ninst * sizeof(InstState), cudaMemcpyHostToDevice));
    StepScalars sc;
    std::memset(&sc, 0, sizeof sc);
    sc.n = (int)ntot;
    sc.n_total = (int)ntot;
    sc.buf = 0;
    sc.rebuild = 1;
    sc.force_rebuild = 1;
    CUDA_TRY(c, cudaMemcpy(c->d_sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
  }
  c->inout = inout;
  c->inoutcounter = 0;
  c->in_part.clear();
  c->next_orig = ntot;
  if (inout) {
    c->class_index.clear();
    for (size_t q = 0; q < c->classes.size(); ++q)
      c->class_index.emplace(std::string((const char*)&c->classes[q], sizeof(PClass)), (int)q);
  }
  c->uploaded = true;
  return PSPH_OK;
}

// ---- in/out-flow boundary (Source/Domain.cpp:1327-1635) ------------------------
// The per-particle work runs in psph_inout.cu; here the reference's ordered
// lists: BC.InPart in its list order, DelPart in index order, AddPart in
// InPart order. A particle's original index orders it as the reference's
// particle array does.

psph_status flow_buffer(psph_ctx* c, size_t bytes) {
  psph_status st;
  if (!c->d_flow_count && (st = dalloc(c, &c->d_flow_count, 4))) return st;
  if (bytes > c->flow_buf_bytes) {
    const size_t cap = std::max(bytes, 2 * c->flow_buf_bytes);
    char* p = nullptr;
    if ((st = dalloc(c, &p, cap))) return st;
    c->d_flow_buf = p;
    c->flow_buf_bytes = cap;
  }
  return PSPH_OK;
}

// slot of every original index of the current order
psph_status flow_slot_map(psph_ctx* c) {
  psph_status st;
  if (c->next_orig > c->slot_cap) {
    const long long cap = std::max(c->next_orig, 2 * c->slot_cap);
    if ((st = dalloc(c, &c->d_slot_of, (size_t)cap))) return st;
    c->slot_cap = cap;
  }
  CUDA_TRY(c, cudaMemsetAsync(c->d_slot_of, 0xff, (size_t)c->next_orig * sizeof(int), c->stream));
  flow_slot_of(view(c), c->h_sc->n, c->d_slot_of, c->stream);
  return PSPH_OK;
}

// the class of a recycled particle, added to the table when new
int flow_class(psph_ctx* c, const PClass& C, bool* added) {
  const std::string key((const char*)&C, sizeof(PClass));
  auto it = c->class_index.find(key);
  if (it != c->class_index.end()) return it->second;
  if ((int)c->classes.size() >= c->cls_cap) return -1;
  const int id = (int)c->classes.size();
  c->classes.push_back(C);
  c->class_index.emplace(key, id);
  *added = true;
  return id;
}

// The fields InFlowBCLeave copies from in-flow particle B into a recycled
// particle (Source/Domain.cpp:1363-1395; T0 and TI are zeroed there).
void flow_copy_fields(PClass& R, const PClass& B) {
  R.material = 1;
  R.p0 = B.p0;
  R.pres_eq = B.pres_eq;
  R.cs = B.cs;
  R.alpha = B.alpha;
  R.beta = B.beta;
  R.mu0 = B.mu0;
  R.mu_ref = B.mu_ref;
  R.t0 = 0.0;
  R.mass = B.mass;
  R.h = B.h;
  R.id = B.id;
  R.ti = 0.0;
  R.rho0 = B.rho0;
  R.shepard = B.shepard;
  R.les = B.les;
  R.csmag = B.csmag;
}

psph_status flow_upload_list(psph_ctx* c, const std::vector<long long>& v) {
  psph_status st;
  if ((st = flow_buffer(c, std::max<size_t>(v.size(), 1) * sizeof(long long)))) return st;
  if (!v.empty())
    CUDA_TRY(c, cudaMemcpyAsync(c->d_flow_buf, v.data(), v.size() * sizeof(long long), cudaMemcpyHostToDevice,
                                c->stream));
  return PSPH_OK;
}

// A user InCon / OutCon on the listed particles (slot and position each):
// called here on the host in list order, the states applied by one launch.
psph_status flow_profile_apply(psph_ctx* c, int which, const std::vector<FlowSlot>& parts, double scale, int set_v,
                               int set_d) {
  std::vector<FlowState> states;
  states.reserve(parts.size());
  for (const FlowSlot& f : parts) {
    if (f.slot < 0) continue;
    const double x[3] = {f.x, f.y, f.z};
    double vel[3] = {0.0, 0.0, 0.0}, den = 0.0;
    c->flow_fn[which](x, vel, &den, c->flow_user[which]);
    states.push_back(FlowState{f.slot, set_v, set_d, 0, scale * vel[0], scale * vel[1], scale * vel[2], den});
  }
  if (states.empty()) return PSPH_OK;
  psph_status st;
  if ((st = flow_buffer(c, states.size() * sizeof(FlowState)))) return st;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_flow_buf, states.data(), states.size() * sizeof(FlowState), cudaMemcpyHostToDevice,
                              c->stream));
  flow_apply(view(c), static_cast<const FlowState*>(c->d_flow_buf), (int)states.size(), c->stream);
  // the host vector must outlive the copy; the buffer is reused by the next list
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return PSPH_OK;
}

// slot and position of the listed original indices (slot -1: not alive)
psph_status flow_gather(psph_ctx* c, const std::vector<long long>& origs, std::vector<FlowSlot>& out) {
  const size_t m = origs.size();
  out.resize(m);
  if (m == 0) return PSPH_OK;
  psph_status st;
  if ((st = flow_buffer(c, m * (sizeof(long long) + sizeof(FlowSlot)) + 64))) return st;
  long long* d_list = static_cast<long long*>(c->d_flow_buf);
  FlowSlot* d_slots =
      reinterpret_cast<FlowSlot*>(static_cast<char*>(c->d_flow_buf) + ((m * sizeof(long long) + 63) & ~size_t(63)));
  CUDA_TRY(c, cudaMemcpyAsync(d_list, origs.data(), m * sizeof(long long), cudaMemcpyHostToDevice, c->stream));
  flow_gather_slots(view(c), d_list, (int)m, c->d_slot_of, d_slots, c->stream);
  CUDA_TRY(c, cudaMemcpyAsync(out.data(), d_slots, m * sizeof(FlowSlot), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return PSPH_OK;
}

// InFlowBCFresh (Source/Domain.cpp:1490-1636), after the step's cell sort
psph_status inout_fresh(psph_ctx* c) {
  const psph_config& k = c->cfgs[0];
  const psph_grid& g = c->grids[0];
  const double cellfac = k.bc_cellfac > 0.0 ? k.bc_cellfac : 3.9;
  const int iof = k.in_out_flow;
  const int n = c->h_sc->n;
  cudaStream_t s = c->stream;
  psph_status st;
  if ((st = flow_slot_map(c))) return st;
  // BC.InPart by the reference's traversal: cells (q2, q3, q1) in loop order,
  // each cell's chain in descending index order
  std::vector<FlowCand> cand;
  auto traverse = [&](int need_io) -> psph_status {
    const int temp1 = (int)std::floor((c->in_loc1 - g.blpf[0]) / g.cell_size[0]);
    psph_status e;
    if ((e = flow_buffer(c, std::max(n, 1) * sizeof(FlowCand)))) return e;
    CUDA_TRY(c, cudaMemsetAsync(c->d_flow_count, 0, sizeof(int), s));
    flow_inflow_candidates(view(c), n, temp1, c->in_loc1, need_io, c->d_flow_count,
                           static_cast<FlowCand*>(c->d_flow_buf), n, s);
    int m = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&m, c->d_flow_count, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(c, cudaStreamSynchronize(s));
    cand.resize((size_t)m);
    if (m > 0)
      CUDA_TRY(c, cudaMemcpy(cand.data(), c->d_flow_buf, (size_t)m * sizeof(FlowCand), cudaMemcpyDeviceToHost));
    std::sort(cand.begin(), cand.end(), [](const FlowCand& a, const FlowCand& b) {
      if (a.cy != b.cy) return a.cy < b.cy;
      if (a.cz != b.cz) return a.cz < b.cz;
      if (a.cx != b.cx) return a.cx < b.cx;
      return a.orig > b.orig;
    });
    c->in_part.clear();
    for (const FlowCand& f : cand) c->in_part.push_back(f.orig);
    return PSPH_OK;
  };
  if (c->inoutcounter == 0) {
    if (iof == 1 || iof == 3) {
      const double* inv = k.in_v;
      if (!(std::sqrt(inv[0] * inv[0] + inv[1] * inv[1] + inv[2] * inv[2]) > 0.0) || !(k.in_density > 0.0))
        return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "BC.inv or BC.inDensity are not defined");
      c->in_loc1 = g.blpf[0] + cellfac * g.hmax;
      if ((st = traverse(0))) return st;
      if (cand.empty()) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "no free particle in the in-flow zone");
      c->in_loc2 = c->in_loc3 = cand[0].x0;
      for (const FlowCand& f : cand) {
        if (f.x0 < c->in_loc2) c->in_loc2 = f.x0;
        if (f.x0 > c->in_loc3) c->in_loc3 = f.x0;
      }
      if ((st = flow_upload_list(c, c->in_part))) return st;
      flow_set_io(view(c), static_cast<const long long*>(c->d_flow_buf), (int)c->in_part.size(), c->d_slot_of, 1, s);
    }
    if (iof == 2 || iof == 3) c->out_loc = g.trpr[0] - cellfac * g.hmax;
    c->inoutcounter = 2;
  }
  if (c->inoutcounter == 1) {
    if ((st = traverse(1))) return st;
    c->inoutcounter = 2;
  }
  int n_out = 0;
  if (iof == 2 || iof == 3) {
    CUDA_TRY(c, cudaMemsetAsync(c->d_flow_count, 0, sizeof(int), s));
    flow_outflow_mark(view(c), n, c->out_loc, c->d_flow_count, s);
    CUDA_TRY(c, cudaMemcpyAsync(&n_out, c->d_flow_count, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(c, cudaStreamSynchronize(s));
  }
  if (!c->in_part.empty()) {  // InCon on BC.InPart
    if (c->flow_fn[PSPH_FLOW_IN]) {
      std::vector<FlowSlot> parts;
      if ((st = flow_gather(c, c->in_part, parts))) return st;
      if ((st = flow_profile_apply(c, PSPH_FLOW_IN, parts, 1.0, 1, 1))) return st;
    } else {
      if ((st = flow_upload_list(c, c->in_part))) return st;
      flow_inflow_state(view(c), static_cast<const long long*>(c->d_flow_buf), (int)c->in_part.size(),
                        c->d_slot_of, k.in_v, k.in_density, s);
    }
  }
  if (n_out > 0) {  // OutCon on BC.OutPart
    const double temp11 = k.mass_conservation ? c->in_part.size() * 1.0 / (n_out * 1.0) : 1.0;
    const double* ov = k.out_v;
    const int set_v = (std::sqrt(ov[0] * ov[0] + ov[1] * ov[1] + ov[2] * ov[2]) > 0.0 || temp11 != 1.0) ? 1 : 0;
    const int set_d = k.out_density > 0.0 ? 1 : 0;
    if (c->flow_fn[PSPH_FLOW_OUT]) {
      std::vector<FlowSlot> parts((size_t)n_out);
      if ((st = flow_buffer(c, (size_t)n_out * sizeof(FlowSlot)))) return st;
      CUDA_TRY(c, cudaMemsetAsync(c->d_flow_count, 0, sizeof(int), s));
      flow_outflow_list(view(c), n, c->out_loc, c->d_flow_count, static_cast<FlowSlot*>(c->d_flow_buf), n_out, s);
      int m = 0;
      CUDA_TRY(c, cudaMemcpyAsync(&m, c->d_flow_count, sizeof(int), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(c, cudaStreamSynchronize(s));
      parts.resize((size_t)std::min(m, n_out));
      if (!parts.empty())
        CUDA_TRY(c, cudaMemcpy(parts.data(), c->d_flow_buf, parts.size() * sizeof(FlowSlot), cudaMemcpyDeviceToHost));
      std::sort(parts.begin(), parts.end(), [](const FlowSlot& a, const FlowSlot& b) { return a.orig < b.orig; });
      if ((st = flow_profile_apply(c, PSPH_FLOW_OUT, parts, temp11, set_v, set_d))) return st;
    } else {
      const double vel[3] = {temp11 * ov[0], temp11 * ov[1], temp11 * ov[2]};
      flow_outflow_state(view(c), n, c->out_loc, vel, k.out_density, set_v, set_d, s);
    }
  }
  CUDA_TRY(c, cudaGetLastError());
  return PSPH_OK;
}

// InFlowBCLeave (Source/Domain.cpp:1327-1488), after the step's update
psph_status inout_leave(psph_ctx* c) {
  const psph_config& k = c->cfgs[0];
  const int iof = k.in_out_flow;
  const int n = c->h_sc->n;
  cudaStream_t s = c->stream;
  psph_status st;
  // DelPart: the particles outside the grid box, in index order
  if ((st = flow_buffer(c, std::max(n, 1) * sizeof(FlowSlot)))) return st;
  CUDA_TRY(c, cudaMemsetAsync(c->d_flow_count, 0, sizeof(int), s));
  flow_leaving(view(c), n, c->d_flow_count, static_cast<FlowSlot*>(c->d_flow_buf), n, s);
  int ndel = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&ndel, c->d_flow_count, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(c, cudaStreamSynchronize(s));
  std::vector<FlowSlot> del((size_t)ndel);
  if (ndel > 0) CUDA_TRY(c, cudaMemcpy(del.data(), c->d_flow_buf, (size_t)ndel * sizeof(FlowSlot), cudaMemcpyDeviceToHost));
  std::sort(del.begin(), del.end(), [](const FlowSlot& a, const FlowSlot& b) { return a.orig < b.orig; });
  // AddPart: in-flow particles past InFlowLoc1, in BC.InPart order
  std::vector<FlowSlot> add;
  std::vector<long long> released;
  if ((iof == 1 || iof == 3) && !c->in_part.empty()) {
    std::vector<FlowSlot> cur;
    if ((st = flow_gather(c, c->in_part, cur))) return st;
    std::vector<long long> keep;
    for (const FlowSlot& f : cur) {
      if (f.slot >= 0 && f.x > c->in_loc1) {
        FlowSlot a = f;
        a.x -= (c->in_loc3 - c->in_loc2 + k.initial_dist);
        add.push_back(a);
        released.push_back(f.orig);
      } else {
        keep.push_back(f.orig);
      }
    }
    c->in_part.swap(keep);
    if (!released.empty()) {
      if ((st = flow_upload_list(c, released))) return st;
      flow_set_io(view(c), static_cast<const long long*>(c->d_flow_buf), (int)released.size(), c->d_slot_of, 0, s);
    }
  }
  const size_t nadd = add.size(), nd = del.size();
  std::vector<FlowRecycle> cmds;
  bool added = false;
  const size_t nreuse = std::min(nadd, nd);
  for (size_t i = 0; i < nreuse; ++i) {  // a freed slot takes the new in-flow particle
    PClass R = c->classes[(size_t)del[i].cls];
    flow_copy_fields(R, c->classes[(size_t)add[i].cls]);
    const int cls = flow_class(c, R, &added);
    if (cls < 0) return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow: too many distinct particle parameter sets");
    FlowRecycle r{del[i].slot, add[i].slot, cls, 0, del[i].orig, add[i].x, add[i].y, add[i].z, 0.0};
    cmds.push_back(r);
    c->in_part.push_back(del[i].orig);
  }
  int appended = 0;
  for (size_t i = nd; i < nadd; ++i) {  // surplus: new particles (the Particle constructor's defaults)
    const PClass& B = c->classes[(size_t)add[i].cls];
    PClass R;
    std::memset(&R, 0, sizeof R);
    R.fpmassc = 1.0;
    R.bm = 300.0;
    R.tin = 4.0;
    R.is_free = 1;
    flow_copy_fields(R, B);
    R.vol = B.mass / B.rho0;
    const int cls = flow_class(c, R, &added);
    if (cls < 0) return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow: too many distinct particle parameter sets");
    const int slot = n + appended;
    if (slot >= c->ncap)
      return set_err(c, PSPH_ERR_UNSUPPORTED, "in/out-flow: the recycled in-flow exceeds the particle headroom (%d)",
                     c->ncap);
    const long long orig = c->next_orig++;
    FlowRecycle r{slot, add[i].slot, cls, 1, orig, add[i].x, add[i].y, add[i].z, B.rho0};
    cmds.push_back(r);
    c->in_part.push_back(orig);
    ++appended;
  }
  if (nadd < nd) c->inoutcounter = 1;  // the surplus slots are deleted (the next sort drops them)
  if (added) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_cls, c->classes.data(), c->classes.size() * sizeof(PClass), cudaMemcpyHostToDevice, s));
    launch_class_constants(c->d_cls, (int)c->classes.size(), c->opt.dim, s);
  }
  if (!cmds.empty()) {
    if ((st = flow_buffer(c, cmds.size() * sizeof(FlowRecycle)))) return st;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_flow_buf, cmds.data(), cmds.size() * sizeof(FlowRecycle), cudaMemcpyHostToDevice, s));
    flow_recycle(view(c), static_cast<const FlowRecycle*>(c->d_flow_buf), (int)cmds.size(), s);
  }
  if (appended > 0) {
    const int nn = n + appended, nt = c->h_sc->n_total + appended;
    CUDA_TRY(c, cudaMemcpyAsync(&c->d_sc->n, &nn, sizeof(int), cudaMemcpyHostToDevice, s));
    CUDA_TRY(c, cudaMemcpyAsync(&c->d_sc->n_total, &nt, sizeof(int), cudaMemcpyHostToDevice, s));
  }
  CUDA_TRY(c, cudaStreamSynchronize(s));
  CUDA_TRY(c, cudaGetLastError());
  return PSPH_OK;
}

// StartAcceleration's a = Gravity and dDensity = 0 (Source/Domain.cpp:1005-1007),
// what a GeneralBefore hook finds
__global__ void start_accel_kernel(double4_32a* __restrict__ A4, const StepScalars* sc, double gx, double gy,
                                   double gz) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < sc->n) A4[s] = make_double4_32a(gx, gy, gz, 0.0);
}

// The FP32 offsets from the cell origins after a GeneralBefore hook moved
// particles (the cell sort's rule; the cells stay those of the sort)
__global__ void offsets32_kernel(DevView v) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  const Persist& P = cur_persist(v);
  const double4_32a xs = P.X4[s];
  const PClass& C = v.cls[P.cls[s]];
  const float h = (float)C.h;
  const int cell = v.S.cellid[s];
  if (cell >= 0) {
    const GridDev& g = grid_of(v, C.inst);
    const int lk = cell - g.cell_base;
    const int cx = lk % g.nc[0], t = lk / g.nc[0], cy = t % g.nc[1], cz = t / g.nc[1];
    v.S.OFF32[s] = make_float4((float)(xs.x - (g.blpf[0] + cx * g.cell_size[0])),
                               (float)(xs.y - (g.blpf[1] + cy * g.cell_size[1])),
                               (float)(v.o.dim == 3 ? xs.z - (g.blpf[2] + cz * g.cell_size[2]) : 0.0), h);
  } else {
    v.S.OFF32[s] = make_float4((float)xs.x, (float)xs.y, (float)xs.z, h);
  }
}

psph_status run_hook(psph_ctx* c, int where) {
  psph_status st;
  if ((st = sync_scalars(c))) return st;
  c->in_hook = where;
  const int rc = c->hook_fn(c, where, c->hook_user);
  c->in_hook = 0;
  if (rc != 0)
    return set_err(c, PSPH_ERR_STATE, "the %s hook asked to stop the run (returned %d)",
                   where == PSPH_HOOK_BEFORE ? "GeneralBefore" : "GeneralAfter", rc);
  return PSPH_OK;
}

// Steps launched in parts, with host work between them (no graph: the host
// decides between the parts): the in/out-flow lists (InFlowBCFresh after the
// cell sort, InFlowBCLeave after the update) and the host hooks (GeneralBefore
// after the neighbour search, GeneralAfter after the forces and the time-step
// bound), in Solve's order (Source/Domain.cpp:1764-1792). With output set, the
// first step writes the snapshot where Solve does, after GeneralAfter.
psph_status split_steps(psph_ctx* c, int64_t nsteps, long long* launched, bool output) {
  psph_status st;
  const bool before = c->hook_fn && (c->hook_mask & PSPH_HOOK_BEFORE);
  const bool after = c->hook_fn && (c->hook_mask & PSPH_HOOK_AFTER);
  for (int64_t k = 0; k < nsteps; ++k) {
    cudaStream_t s = c->stream;
    launch_begin(view(c), s);
    launch_sort(view(c), s);
    CUDA_TRY(c, cudaGetLastError());
    if ((st = sync_scalars(c))) return st;
    if (c->h_sc->all_stop) break;
    if (c->inout && (st = inout_fresh(c))) return st;
    launch_nlist(view(c), s);
    if (c->opt.skin > 0.f) launch_skin_offsets(view(c), s);
    if (before) {
      const int n = c->h_sc->n;
      const double* gv = c->opt.gravity;
      start_accel_kernel<<<n > 0 ? (n + 255) / 256 : 1, 256, 0, s>>>(c->S.A4, c->d_sc, gv[0], gv[1], gv[2]);
      c->hook_set_a = c->hook_set_x = false;
      if ((st = run_hook(c, PSPH_HOOK_BEFORE))) return st;
      c->opt.a_from_hook = c->hook_set_a ? 1 : 0;
      if (c->hook_set_x) offsets32_kernel<<<n > 0 ? (n + 255) / 256 : 1, 256, 0, s>>>(view(c));
    }
    {
      const DevView v = view(c);
      if (v.o.fp32) launch_prepare32(v, s);
      else launch_prepare(v, s);
      if (v.o.couple_soil && v.o.swi != 2) launch_saturation(v, s);
      if (v.o.fsi) launch_fsi(v, s);
      if (v.o.fp32) launch_forces32(v, s);
      else launch_forces(v, s);
      if (v.o.mixed) launch_coupling(v, s);
      if (v.o.closure) launch_closure(v, s);
      launch_dt(v, s);
    }
    c->opt.a_from_hook = 0;
    if (after && (st = run_hook(c, PSPH_HOOK_AFTER))) return st;
    if (output && k == 0) {  // Solve's output point (Source/Domain.cpp:1773-1788)
      std::string e;
      const int hi = c->inout ? (int)c->next_orig : (int)c->inst_off[1];
      if (!output_gather(c->out, view(c), 0, hi, s, &e)) return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
    }
    {
      const DevView v = view(c);
      launch_update(v, s);
      launch_end(v, s);
      CUDA_TRY(c, cudaGetLastError());
      *launched += launches_per_step(v);
    }
    if (output && k == 0) {
      std::string e;
      const char* names[3] = {c->out_names[0].c_str(), c->out_names[1].c_str(), c->out_names[2].c_str()};
      if (!output_commit(c->out, c->out_key.c_str(), names, nullptr, 0, &e))
        return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
      *launched += 4;
    }
    if ((st = sync_scalars(c))) return st;
    if (c->h_sc->status) break;
    if (c->inout && (st = inout_leave(c))) return st;
  }
  return sync_scalars(c);
}

psph_status step_impl(psph_ctx* c, int64_t nsteps, const double* t_stop, double t_all, int64_t* steps_done) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  if (steps_done)
    for (int q = 0; q < c->ninst; ++q) steps_done[q] = 0;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_step before psph_upload");
  psph_status st;
  if (nsteps <= 0) return c->timing ? PSPH_OK : build_graph(c);
  if ((st = arm(c, t_stop, t_all))) return st;
  std::vector<long long> steps0(c->ninst);
  for (int q = 0; q < c->ninst; ++q) steps0[q] = c->h_inst[q].steps;
  for (int e = 0; e < kNumPhases; ++e) c->phase_ms[e] = 0.0;
  long long launched = 0;
  if (c->out_requested && (c->inout || c->hook_fn)) {
    c->out_requested = false;
    if ((st = split_steps(c, nsteps, &launched, true))) return st;
    nsteps = 0;
  } else if (c->out_requested) {
    // the output step: launched directly, the snapshot gathered between its
    // forces and its update; its copy to the host and the file writes overlap
    // the steps that follow
    c->out_requested = false;
    std::string e;
    bool ok = true;
    enqueue_step(c, [&] { ok = output_gather(c->out, view(c), 0, (int)c->inst_off[1], c->stream, &e); });
    CUDA_TRY(c, cudaGetLastError());
    if (!ok) return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
    const char* names[3] = {c->out_names[0].c_str(), c->out_names[1].c_str(), c->out_names[2].c_str()};
    if (!output_commit(c->out, c->out_key.c_str(), names, nullptr, 0, &e))
      return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
    launched += launches_per_step(view(c)) + 4;
    if ((st = sync_scalars(c))) return st;
    --nsteps;
    if (c->h_sc->all_stop || c->h_sc->status) nsteps = 0;
  }
  if (nsteps <= 0) {
  } else if (c->inout || c->hook_fn) {
    if ((st = split_steps(c, nsteps, &launched, false))) return st;
  } else if (c->timing) {
    for (int64_t s = 0; s < nsteps; ++s) {
      enqueue_step(c);
      CUDA_TRY(c, cudaGetLastError());
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      for (int e = 0; e < kNumPhases; ++e) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[e], c->ev[e + 1]);
        c->phase_ms[e] += ms;
      }
      launched += launches_per_step(view(c));
      if ((st = sync_scalars(c))) return st;
      if (c->h_sc->all_stop) break;
    }
  } else {
    if ((st = build_graph(c))) return st;
    int64_t left = nsteps;
    while (left > 0) {
      const int64_t chunk = std::min<int64_t>(left, 256);
      for (int64_t s = 0; s < chunk; ++s) CUDA_TRY(c, cudaGraphLaunch(c->graph, c->stream));
      left -= chunk;
      launched += chunk * launches_per_step(view(c));
      if ((st = sync_scalars(c))) return st;
      if (c->h_sc->all_stop || c->h_sc->status) break;
    }
  }
  if ((st = sync_scalars(c))) return st;
  if (steps_done)
    for (int q = 0; q < c->ninst; ++q) steps_done[q] = c->h_inst[q].steps - steps0[q];
  c->last_launches = launched;
  const uint32_t status = c->h_sc->status;
  // the root cause first: a non-finite state also throws particles off the grid
  if (status & ST_NONFINITE) return set_err(c, PSPH_ERR_NONFINITE, "non-finite acceleration or density rate");
  if (status & ST_DT_COLLAPSE)
    return set_err(c, PSPH_ERR_DT_COLLAPSE,
                   "Too small time step, please choose a smaller time step initially to make the simulation more stable");
  if (status & ST_OUT_OF_GRID)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "a particle lies more than hmax outside the cell grid");
  // a bounded device-side wait that gave up (the kernel finished its work
  // without the data it waited for and reported it)
  if (status & ST_CLOSURE_TIMEOUT)
    return set_err(c, PSPH_ERR_CUDA, "the closure kernel's tensor-core completion wait gave up");
  if (status & ST_STAGE_TIMEOUT)
    return set_err(c, PSPH_ERR_CUDA, "the neighbour scan's shared-memory staging wait gave up");
  if (status & ST_LIST_MISMATCH)
    return set_err(c, PSPH_ERR_CUDA, "a pair inside the kernel support is missing from its partner's list");
  return PSPH_OK;
}

// Alive particles of instance q in original order: (original index, slot).
// Slots flagged by the last update as leaving stay out (the next sort drops them).
psph_status alive_of(psph_ctx* c, int q, std::vector<std::pair<int, int>>& order, std::vector<int>* cls_out) {
  psph_status st;
  if ((st = sync_scalars(c))) return st;
  const StepScalars sc = *c->h_sc;
  const size_t n = (size_t)sc.n;
  const Persist& P = sc.buf ? c->PB : c->PA;
  std::vector<uint8_t> alive(n);
  std::vector<int> orig(n);
  CUDA_TRY(c, cudaMemcpy(alive.data(), c->d_alive, n, cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(orig.data(), P.orig, n * sizeof(int), cudaMemcpyDeviceToHost));
  if (cls_out) {
    cls_out->resize(n);
    CUDA_TRY(c, cudaMemcpy(cls_out->data(), P.cls, n * sizeof(int), cudaMemcpyDeviceToHost));
  }
  // original indices are unique: place each alive slot at its original index
  // (a counting sort, linear in n) instead of sorting the pairs
  const int64_t lo = c->inst_off[q], hi = c->inst_off[q + 1];
  std::vector<int> slot_of((size_t)(hi - lo), -1);
  for (size_t s = 0; s < n; ++s)
    if (alive[s] && orig[s] >= lo && orig[s] < hi) slot_of[(size_t)(orig[s] - lo)] = (int)s;
  order.clear();
  order.reserve(slot_of.size());
  for (size_t k = 0; k < slot_of.size(); ++k)
    if (slot_of[k] >= 0) order.emplace_back((int)(lo + (int64_t)k), slot_of[k]);
  return PSPH_OK;
}

// Download on the device: each sorted particle's output row (its rank by
// original index among the instance's alive particles, Array::DelItems'
// order), then per requested field one gather into a staging buffer laid out
// as the caller's array and one copy into that array.
__global__ void dl_flag_kernel(const uint8_t* __restrict__ alive, const int* __restrict__ orig, int n, int lo,
                               int hi, int* __restrict__ flag) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n && alive[s] && orig[s] >= lo && orig[s] < hi) flag[orig[s] - lo] = 1;
}
__global__ void dl_row_kernel(const uint8_t* __restrict__ alive, const int* __restrict__ orig, int n, int lo, int hi,
                              const int* __restrict__ rank, int* __restrict__ row) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) row[s] = (alive[s] && orig[s] >= lo && orig[s] < hi) ? rank[orig[s] - lo] : -1;
}
// dst[row * width + e] = src[s * stride + off + e]
__global__ void dl_gather_kernel(const double* __restrict__ src, int stride, int off, int width,
                                 double* __restrict__ dst, const int* __restrict__ row, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r < 0) return;
  for (int e = 0; e < width; ++e) dst[(size_t)r * width + e] = src[(size_t)s * stride + off + e];
}
// psph_patch: the caller's row r = row[s] back into slot s (dl_gather_kernel's reverse)
__global__ void patch_scatter_kernel(double* __restrict__ dst, int stride, int off, int width,
                                     const double* __restrict__ src, const int* __restrict__ row, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r < 0) return;
  for (int e = 0; e < width; ++e) dst[(size_t)s * stride + off + e] = src[(size_t)r * width + e];
}
__global__ void patch_scatter_int_kernel(int* __restrict__ dst, const int* __restrict__ src,
                                         const int* __restrict__ row, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r >= 0) dst[s] = src[r];
}
// a per-particle int per row
__global__ void dl_gather_int_kernel(const int* __restrict__ src, int* __restrict__ dst, const int* __restrict__ row,
                                     int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r >= 0) dst[r] = src[s];
}
// original index (relative to the instance) per row
__global__ void dl_orig_kernel(const int* __restrict__ orig, long long base, long long* __restrict__ dst,
                               const int* __restrict__ row, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r >= 0) dst[r] = orig[s] - base;
}
// a class constant (int or double at byte offset off of PClass) per row
__global__ void dl_class_kernel(const PClass* __restrict__ tab, const int* __restrict__ cls, size_t off, int is_int,
                                void* __restrict__ dst, const int* __restrict__ row, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int r = row[s];
  if (r < 0) return;
  const char* rec = reinterpret_cast<const char*>(tab + cls[s]) + off;
  if (is_int) static_cast<int32_t*>(dst)[r] = *reinterpret_cast<const int*>(rec);
  else static_cast<double*>(dst)[r] = *reinterpret_cast<const double*>(rec);
}

// Output rows of instance q on the device: c->dl_row[s] is slot s's row in
// original order (leavers and other instances: -1); *m receives the row count.
psph_status download_rows(psph_ctx* c, int q, int64_t* m) {
  psph_status st;
  if ((st = sync_scalars(c))) return st;
  const int n = c->h_sc->n;
  const Persist& P = c->h_sc->buf ? c->PB : c->PA;
  cudaStream_t s = c->stream;
  const size_t N = (size_t)c->ncap;
  // (an in/out-flow domain's appended particles take original indices past the upload's)
  const int lo = (int)c->inst_off[q], hi = c->inout ? (int)c->next_orig : (int)c->inst_off[q + 1], len = hi - lo;
  if (!c->dl_row && (st = dalloc(c, &c->dl_row, N))) return st;
  if ((size_t)len + 1 > c->dl_cap) {  // the per-original-index scan (grows with an in/out-flow domain)
    const size_t cap = std::max((size_t)len + 1, std::max(N + 1, 2 * c->dl_cap));
    if ((st = dalloc(c, &c->dl_flag, cap)) || (st = dalloc(c, &c->dl_rank, cap)) ||
        (st = dalloc(c, &c->dl_bs, cap / 1024 + 2)))
      return st;
    c->dl_cap = cap;
  }
  const int nb = n > 0 ? (n + 255) / 256 : 1;
  CUDA_TRY(c, cudaMemsetAsync(c->dl_flag, 0, sizeof(int) * (size_t)(len + 1), s));
  if (n > 0) dl_flag_kernel<<<nb, 256, 0, s>>>(c->d_alive, P.orig, n, lo, hi, c->dl_flag);
  launch_exclusive_scan(c->dl_flag, c->dl_rank, len, c->dl_bs, s);
  if (n > 0) dl_row_kernel<<<nb, 256, 0, s>>>(c->d_alive, P.orig, n, lo, hi, c->dl_rank, c->dl_row);
  int m32 = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&m32, c->dl_rank + len, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(c, cudaStreamSynchronize(s));
  *m = m32;
  return PSPH_OK;
}

psph_status download_impl(psph_ctx* c, int q, psph_particles* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_download before psph_upload");
  if (q < 0 || q >= c->ninst) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "instance %d out of range", q);
  psph_status st;
  int64_t m = 0;
  if ((st = download_rows(c, q, &m))) return st;
  const int n = c->h_sc->n;
  const Persist& P = c->h_sc->buf ? c->PB : c->PA;
  const Options& o = c->opt;
  const bool lf = (o.scheme == PSPH_LEAPFROG);
  cudaStream_t s = c->stream;
  const size_t N = (size_t)c->ncap;
  const int nb = n > 0 ? (n + 255) / 256 : 1;
  if (out->n < m)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "output holds %lld particles, need %lld", (long long)out->n, (long long)m);
  out->n = m;
  if (m == 0) return PSPH_OK;

  // (destination, source, source stride, offset, width)
  struct F { double* out; const double* dev; int stride, off, width; };
  auto d4 = [](const double4_32a* p) { return reinterpret_cast<const double*>(p); };
  const F fields[] = {
      {out->x, d4(P.X4), 4, 0, 3}, {out->density, d4(P.X4), 4, 3, 1},
      {out->v, d4(P.V4), 4, 0, 3}, {out->pressure, d4(P.V4), 4, 3, 1},
      {lf ? out->va : out->vb, d4(P.H4), 4, 0, 3}, {lf ? out->densitya : out->densityb, d4(P.H4), 4, 3, 1},
      {lf ? out->vb : nullptr, d4(P.H4b), 4, 0, 3}, {lf ? out->densityb : nullptr, d4(P.H4b), 4, 3, 1},
      {out->a, d4(c->S.A4), 4, 0, 3}, {out->ddensity, d4(c->S.A4), 4, 3, 1},
      {out->nsv, d4(c->S.nsv4), 4, 0, 3}, {out->vxsph, d4(c->S.vxsph4), 4, 0, 3},
      {out->zwab, c->S.zwab, 1, 0, 1}, {out->sumden, c->S.sumden, 1, 0, 1}, {out->sumkernel, c->S.sumkernel, 1, 0, 1},
      {out->shear_rate, c->S.shear_rate, 1, 0, 1}, {out->sbar, c->S.sbar, 1, 0, 1},
      {out->mu, o.dyn_mu ? P.mu : nullptr, 1, 0, 1},
      {out->strain_rate, c->S.strain_rate, 9, 0, 9}, {out->rotation_rate, c->S.rotation_rate, 9, 0, 9},
      {out->sigma, P.sigma, 9, 0, 9}, {out->strain, P.strain, 9, 0, 9}, {out->shear_stress, P.shear, 9, 0, 9},
      {out->tir, P.tir, 9, 0, 9}, {out->s, c->S.s_acc, 1, 0, 1},
      {lf ? out->sigmaa : out->sigmab, P.sigma_h, 9, 0, 9}, {lf ? out->sigmab : nullptr, c->S.sigma_o, 9, 0, 9},
      {lf ? out->straina : out->strainb, P.strain_h, 9, 0, 9}, {lf ? out->strainb : nullptr, c->S.strain_o, 9, 0, 9},
      {lf ? out->shear_stressa : out->shear_stressb, P.shear_h, 9, 0, 9},
      {lf ? out->shear_stressb : nullptr, c->S.shear_o, 9, 0, 9},
  };
  // The requested fields are gathered into the device staging buffer in
  // batches of at most kStageWidth values per row (a wider field alone); the
  // first batch's gathers run while host threads populate the output pages.
  constexpr int kStageWidth = 16;
  std::vector<const F*> act;
  int width = 1;
  for (const F& f : fields)
    if (f.out && f.dev) {
      act.push_back(&f);
      width = std::max(width, f.width);
    }
  std::vector<int> batch_of(act.size()), seg(act.size());
  int stage = width, nbatch = 0;
  for (size_t a = 0, used = 0; a < act.size(); ++a) {
    if (used > 0 && used + act[a]->width > (size_t)std::max(kStageWidth, width)) {
      ++nbatch;
      used = 0;
    }
    batch_of[a] = nbatch;
    seg[a] = (int)used;
    used += act[a]->width;
    stage = std::max(stage, (int)used);
  }
  if (!act.empty()) ++nbatch;
  if (stage > c->dl_width) {
    if ((st = dalloc(c, &c->dl_buf, N * (size_t)stage))) return st;
    c->dl_width = stage;
  }
  auto gather_batch = [&](int b) {
    for (size_t a = 0; a < act.size(); ++a) {
      if (batch_of[a] != b) continue;
      const F& f = *act[a];
      // the FP32C fluid kernel keeps its strain-rate sums in FP32: expand them first
      if (f.dev == c->S.strain_rate && c->S.sr32) launch_expand_sr32(view(c), n, s);
      dl_gather_kernel<<<nb, 256, 0, s>>>(f.dev, f.stride, f.off, f.width, c->dl_buf + (size_t)seg[a] * m,
                                          c->dl_row, n);
    }
  };
  if (nbatch > 0) gather_batch(0);
  {
    // Fresh output pages are populated here by host threads in parallel (one
    // write per page; the copies overwrite them): a device copy into
    // untouched pageable memory would take each page fault in turn.
    std::vector<std::pair<char*, size_t>> ranges;
    for (const F* f : act) ranges.emplace_back(reinterpret_cast<char*>(f->out), (size_t)m * f->width * sizeof(double));
    size_t total = 0;
    for (const auto& r : ranges) total += r.second;
    const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
    const int nth = host_threads((int64_t)(total / 64));
    if (nth > 1)
      run_threads(nth, [&](int t) {
        for (const auto& r : ranges) {
          const size_t a = r.second * t / nth, b = r.second * (t + 1) / nth;
          for (size_t off = a; off < b; off += page) reinterpret_cast<volatile char*>(r.first)[off] = 0;
        }
      });
  }
  for (int b = 0; b < nbatch; ++b) {
    if (b > 0) gather_batch(b);  // after the previous batch's copies (same stream)
    for (size_t a = 0; a < act.size(); ++a) {
      if (batch_of[a] != b) continue;
      CUDA_TRY(c, cudaMemcpyAsync(act[a]->out, c->dl_buf + (size_t)seg[a] * m,
                                  (size_t)m * act[a]->width * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
  }
  if (out->in_out && P.io) {  // Particle::InOut (in/out-flow domains)
    int* dst = reinterpret_cast<int*>(c->dl_buf);
    dl_gather_int_kernel<<<nb, 256, 0, s>>>(P.io, dst, c->dl_row, n);
    CUDA_TRY(c, cudaMemcpyAsync(out->in_out, dst, (size_t)m * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  }
  // class constants, gathered from the device class table
  struct K { void* out; size_t off; int is_int; };
  const K consts[] = {
      {out->id, offsetof(PClass, id), 1}, {out->material, offsetof(PClass, material), 1},
      {out->is_free, offsetof(PClass, is_free), 1}, {out->no_slip, offsetof(PClass, no_slip), 1},
      {out->pres_eq, offsetof(PClass, pres_eq), 1}, {out->shepard, offsetof(PClass, shepard), 1},
      {out->les, offsetof(PClass, les), 1}, {out->vis_m, offsetof(PClass, vis_m), 1},
      {out->fail, offsetof(PClass, fail), 1},
      {out->mass, offsetof(PClass, mass), 0}, {out->h, offsetof(PClass, h), 0}, {out->cs, offsetof(PClass, cs), 0},
      {out->p0, offsetof(PClass, p0), 0}, {out->ref_density, offsetof(PClass, rho0), 0},
      {out->fpmassc, offsetof(PClass, fpmassc), 0}, {out->alpha, offsetof(PClass, alpha), 0},
      {out->beta, offsetof(PClass, beta), 0}, {o.dyn_mu ? nullptr : out->mu, offsetof(PClass, mu0), 0},
      {out->mu_ref, offsetof(PClass, mu_ref), 0}, {out->t0, offsetof(PClass, t0), 0},
      {out->bingham_m, offsetof(PClass, bm), 0}, {out->csmag, offsetof(PClass, csmag), 0},
      {out->ti, offsetof(PClass, ti), 0}, {out->tin, offsetof(PClass, tin), 0},
      {out->ti_init_dist, offsetof(PClass, tid), 0}, {out->g_mod, offsetof(PClass, g_mod), 0},
      {out->k_mod, offsetof(PClass, k_mod), 0}, {out->sigmay, offsetof(PClass, sigmay), 0},
      {out->cohesion, offsetof(PClass, coh), 0}, {out->phi, offsetof(PClass, phi), 0},
      {out->psi, offsetof(PClass, psi), 0},
      {out->seepage_type, offsetof(PClass, seep_type), 1}, {out->var_porosity, offsetof(PClass, var_por), 1},
      {out->is_sat, offsetof(PClass, is_sat), 1}, {out->n0, offsetof(PClass, n0), 0},
      {out->d, offsetof(PClass, dgrain), 0}, {out->rho_f, offsetof(PClass, rho_f), 0},
      {out->volume, offsetof(PClass, vol), 0},
  };
  for (const K& k : consts) {
    if (!k.out) continue;
    dl_class_kernel<<<nb, 256, 0, s>>>(c->d_cls, P.cls, k.off, k.is_int, c->dl_buf, c->dl_row, n);
    CUDA_TRY(c, cudaMemcpyAsync(k.out, c->dl_buf, (size_t)m * (k.is_int ? sizeof(int32_t) : sizeof(double)),
                                cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(c, cudaStreamSynchronize(s));
  CUDA_TRY(c, cudaGetLastError());
  return PSPH_OK;
}

psph_status integrator_impl(psph_ctx* c, int q, psph_integrator* it) {
  if (!c || !it) return PSPH_ERR_INVALID_ARGUMENT;
  if (q < 0 || q >= c->ninst) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "instance %d out of range", q);
  if (!c->uploaded) {
    *it = c->integ[q];
    return PSPH_OK;
  }
  psph_status st = sync_scalars(c);
  if (st) return st;
  const InstState& s = c->h_inst[q];
  it->time = s.time;
  it->deltat = s.deltat;
  it->deltatint = s.deltatint;
  it->deltatmin = s.deltatmin;
  it->steps = s.steps;
  it->first_step = s.first_step;
  it->ct = s.ct;
  it->shepard_counter = s.shepard_counter;
  it->pad = 0;
  return PSPH_OK;
}

// (the rows are counted on the device: the alive flags and original indices
// of millions of particles stay there)
// The per-particle parameters psph_patch reads, over a particle's current
// parameter set (the conversions of psph_upload; k and k2 are read on upload
// only, as psph_download leaves them).
void class_overlay(PClass& C, const psph_particles* p, int64_t i, bool dyn_mu) {
  auto d = [&](const double* a, double& f) {
    if (a) f = a[i];
  };
  auto n = [&](const int32_t* a, int& f) {
    if (a) f = a[i];
  };
  d(p->cs, C.cs); d(p->p0, C.p0); d(p->ref_density, C.rho0); d(p->fpmassc, C.fpmassc);
  d(p->alpha, C.alpha); d(p->beta, C.beta);
  if (!dyn_mu) d(p->mu, C.mu0);
  d(p->mu_ref, C.mu_ref); d(p->t0, C.t0); d(p->bingham_m, C.bm); d(p->csmag, C.csmag); d(p->ti, C.ti);
  d(p->tin, C.tin); d(p->ti_init_dist, C.tid); d(p->g_mod, C.g_mod); d(p->k_mod, C.k_mod); d(p->sigmay, C.sigmay);
  d(p->cohesion, C.coh); d(p->phi, C.phi); d(p->psi, C.psi); d(p->h, C.h); d(p->mass, C.mass);
  n(p->material, C.material); n(p->pres_eq, C.pres_eq); n(p->vis_m, C.vis_m); n(p->fail, C.fail); n(p->id, C.id);
  auto b = [&](const int32_t* a, int& f) {
    if (a) f = a[i] != 0;
  };
  b(p->is_free, C.is_free); b(p->no_slip, C.no_slip); b(p->shepard, C.shepard); b(p->les, C.les);
  if (C.material == 3) {
    n(p->seepage_type, C.seep_type);
    b(p->var_porosity, C.var_por);
    b(p->is_sat, C.is_sat);
    d(p->n0, C.n0); d(p->d, C.dgrain); d(p->rho_f, C.rho_f); d(p->volume, C.vol);
  }
}

psph_status patch_impl(psph_ctx* c, const psph_particles* p) {
  if (!c || !p) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_patch before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "psph_patch applies to single-domain contexts");
  psph_status st;
  int64_t m = 0;
  if ((st = download_rows(c, 0, &m))) return st;
  if (p->n != m)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "psph_patch got %lld particles, the context holds %lld",
                   (long long)p->n, (long long)m);
  if (m == 0) return PSPH_OK;
  const int n = c->h_sc->n;
  const Persist& P = c->h_sc->buf ? c->PB : c->PA;
  const Options& o = c->opt;
  const bool lf = (o.scheme == PSPH_LEAPFROG);
  cudaStream_t s = c->stream;
  const size_t N = (size_t)c->ncap;
  const int nb = n > 0 ? (n + 255) / 256 : 1;
  // accelerations and density rates at GeneralBefore are the step's starting
  // values: unchanged ones (Gravity, 0) need nothing
  bool set_a = p->a || p->ddensity;
  if (set_a && c->in_hook == PSPH_HOOK_BEFORE) {
    bool same = true;
    for (int64_t r = 0; r < m && same; ++r) {
      if (p->a)
        for (int k = 0; k < 3; ++k) same = same && p->a[3 * r + k] == o.gravity[k];
      if (p->ddensity) same = same && p->ddensity[r] == 0.0;
    }
    if (same) {
      set_a = false;
    } else if (o.fp32) {
      return set_err(c, PSPH_ERR_UNSUPPORTED,
                     "a GeneralBefore hook changed accelerations or density rates: the FP32C pair kernels start "
                     "them from Gravity (use the FP64 form, or psph_config.body_force for a constant acceleration)");
    } else {
      c->hook_set_a = true;
    }
  }
  if (p->x && c->in_hook == PSPH_HOOK_BEFORE) c->hook_set_x = true;
  // with a skin the next step lists again (patched positions may have moved
  // particles past the skin)
  if (c->opt.skin > 0.f) launch_mark_rebuild(view(c), false, true, c->stream);
  struct F { const double* in; double* dev; int stride, off, width; };
  auto d4 = [](double4_32a* q) { return reinterpret_cast<double*>(q); };
  const F fields[] = {
      {p->x, d4(P.X4), 4, 0, 3}, {p->density, d4(P.X4), 4, 3, 1},
      {p->v, d4(P.V4), 4, 0, 3}, {p->pressure, d4(P.V4), 4, 3, 1},
      {lf ? p->va : p->vb, d4(P.H4), 4, 0, 3}, {lf ? p->densitya : p->densityb, d4(P.H4), 4, 3, 1},
      {lf ? p->vb : nullptr, d4(P.H4b), 4, 0, 3}, {lf ? p->densityb : nullptr, d4(P.H4b), 4, 3, 1},
      {set_a ? p->a : nullptr, d4(c->S.A4), 4, 0, 3}, {set_a ? p->ddensity : nullptr, d4(c->S.A4), 4, 3, 1},
      {o.dyn_mu ? p->mu : nullptr, P.mu, 1, 0, 1},
      {p->sigma, P.sigma, 9, 0, 9}, {p->strain, P.strain, 9, 0, 9}, {p->shear_stress, P.shear, 9, 0, 9},
      {lf ? p->sigmaa : p->sigmab, P.sigma_h, 9, 0, 9}, {lf ? p->straina : p->strainb, P.strain_h, 9, 0, 9},
      {lf ? p->shear_stressa : p->shear_stressb, P.shear_h, 9, 0, 9},
  };
  if (c->dl_width < 9) {
    if ((st = dalloc(c, &c->dl_buf, N * 9))) return st;
    c->dl_width = 9;
  }
  for (const F& f : fields) {
    if (!f.in || !f.dev) continue;
    CUDA_TRY(c, cudaMemcpyAsync(c->dl_buf, f.in, (size_t)m * f.width * sizeof(double), cudaMemcpyHostToDevice, s));
    patch_scatter_kernel<<<nb, 256, 0, s>>>(f.dev, f.stride, f.off, f.width, c->dl_buf, c->dl_row, n);
  }
  CUDA_TRY(c, cudaGetLastError());

  // per-particle parameters: each particle's set, found or added
  std::vector<int> cur((size_t)m), next((size_t)m);
  {
    int* dcls = reinterpret_cast<int*>(c->dl_buf);
    dl_gather_int_kernel<<<nb, 256, 0, s>>>(P.cls, dcls, c->dl_row, n);
    CUDA_TRY(c, cudaMemcpyAsync(cur.data(), dcls, (size_t)m * sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(c, cudaStreamSynchronize(s));
  }
  if (c->class_index.empty())
    for (size_t q = 0; q < c->classes.size(); ++q)
      c->class_index.emplace(std::string((const char*)&c->classes[q], sizeof(PClass)), (int)q);
  const size_t ncls0 = c->classes.size();
  bool changed = false;
  int last_in = -1, last_out = -1;
  PClass last_rec;
  std::memset(&last_rec, 0, sizeof last_rec);
  const bool has_params =
      p->cs || p->p0 || p->ref_density || p->fpmassc || p->alpha || p->beta || (!o.dyn_mu && p->mu) || p->mu_ref ||
      p->t0 || p->bingham_m || p->csmag || p->ti || p->tin || p->ti_init_dist || p->g_mod || p->k_mod ||
      p->sigmay || p->cohesion || p->phi || p->psi || p->h || p->mass || p->material || p->pres_eq || p->vis_m ||
      p->fail || p->id || p->is_free || p->no_slip || p->shepard || p->les || p->seepage_type ||
      p->var_porosity || p->is_sat || p->n0 || p->d || p->rho_f || p->volume;
  for (int64_t r = 0; has_params && r < m; ++r) {
    PClass C = c->classes[(size_t)cur[(size_t)r]];
    class_overlay(C, p, r, o.dyn_mu != 0);
    int id;
    if (last_out >= 0 && cur[(size_t)r] == last_in && std::memcmp(&C, &last_rec, sizeof C) == 0) {
      id = last_out;
    } else {
      const std::string key((const char*)&C, sizeof(PClass));
      auto it = c->class_index.find(key);
      if (it != c->class_index.end()) {
        id = it->second;
      } else {
        id = (int)c->classes.size();
        if (id >= 65535) return set_err(c, PSPH_ERR_UNSUPPORTED, "more than 65535 distinct particle parameter sets");
        c->classes.push_back(C);
        c->class_index.emplace(key, id);
      }
      last_in = cur[(size_t)r];
      last_out = id;
      last_rec = C;
    }
    next[(size_t)r] = id;
    changed = changed || id != cur[(size_t)r];
  }
  if (changed) {
    // the step's kernels and buffers were chosen for the parameter sets of the
    // upload: a change that alters any of those choices is refused
    auto refuse = [&](const char* why) {
      c->classes.resize(ncls0);
      c->class_index.clear();
      return set_err(c, PSPH_ERR_UNSUPPORTED, "psph_patch: changed particle parameters %s", why);
    };
    if (o.fp32) return refuse("in the FP32C form");
    if (o.mixed) return refuse("in a domain of two materials");
    int mats0 = 0, mats1 = 0;
    for (size_t q = 0; q < c->classes.size(); ++q) (q < ncls0 ? mats0 : mats1) |= 1 << c->classes[q].material;
    if (mats1 & ~mats0) return refuse("introduce a material the domain did not have");
    for (size_t q = ncls0; q < c->classes.size(); ++q) c->classes[q].inst = 0;
    Options o1 = o;
    derive_class_options(c->classes, false, o.dyn_mu != 0, o1);
    if (o1.uniform_h != o.uniform_h || o1.inv_h != o.inv_h) return refuse("make h differ where it was uniform");
    if (o1.any_av != o.any_av) return refuse("switch on artificial viscosity where no particle had it");
    if (o1.any_ti != o.any_ti) return refuse("switch on tensile instability where no particle had it");
    if (o1.need_sr != o.need_sr) return refuse("ask for strain rates (T0 or LES) where no particle did");
    if (o1.any_shepard != o.any_shepard) return refuse("switch on Shepard filtering where no particle had it");
    if (o1.uniform_eos != o.uniform_eos || o1.eos_cls != o.eos_cls)
      return refuse("give the fluid a second equation of state");
    if (o1.uniform_mu != o.uniform_mu || o1.mu_u != o.mu_u)
      return refuse("change a viscosity every free particle shared");
    // the grown table (each set's derived constants recomputed on the device)
    if ((int)c->classes.size() > c->cls_cap) {
      PClass* grown = nullptr;
      const int cap = std::max((int)c->classes.size(), 2 * c->cls_cap);
      if ((st = dalloc(c, &grown, (size_t)cap))) return st;
      c->d_cls = grown;
      c->cls_cap = cap;
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->d_cls, c->classes.data(), c->classes.size() * sizeof(PClass),
                                cudaMemcpyHostToDevice, s));
    launch_class_constants(c->d_cls, (int)c->classes.size(), o.dim, s);
    c->opt.nclasses = (int)c->classes.size();
    int* dnext = reinterpret_cast<int*>(c->dl_buf);
    CUDA_TRY(c, cudaMemcpyAsync(dnext, next.data(), (size_t)m * sizeof(int), cudaMemcpyHostToDevice, s));
    patch_scatter_int_kernel<<<nb, 256, 0, s>>>(P.cls, dnext, c->dl_row, n);
    if (c->graph) {  // the launches hold the class table: capture the step again
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
    }
  } else if (c->classes.size() > ncls0) {
    c->classes.resize(ncls0);  // sets looked up but unused
    c->class_index.clear();
  }
  CUDA_TRY(c, cudaStreamSynchronize(s));
  CUDA_TRY(c, cudaGetLastError());
  return PSPH_OK;
}

int64_t num_particles_impl(psph_ctx* c, int q) {
  if (!c || !c->uploaded || q < 0 || q >= c->ninst) return 0;
  int64_t m = 0;
  if (download_rows(c, q, &m)) return -1;
  return m;
}

psph_status original_index_impl(psph_ctx* c, int q, int64_t* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_original_index before psph_upload");
  if (q < 0 || q >= c->ninst) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "instance %d out of range", q);
  int64_t m = 0;
  psph_status st = download_rows(c, q, &m);
  if (st) return st;
  if (m == 0) return PSPH_OK;
  const int n = c->h_sc->n;
  const Persist& P = c->h_sc->buf ? c->PB : c->PA;
  if (c->dl_width < 1) {
    if ((st = dalloc(c, &c->dl_buf, (size_t)c->ncap))) return st;
    c->dl_width = 1;
  }
  long long* dst = reinterpret_cast<long long*>(c->dl_buf);
  dl_orig_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(P.orig, c->inst_off[q], dst, c->dl_row, n);
  CUDA_TRY(c, cudaMemcpyAsync(out, dst, (size_t)m * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  CUDA_TRY(c, cudaGetLastError());
  return PSPH_OK;
}

}  // namespace

extern "C" {

int psph_abi_version(void) { return PSPH_ABI_VERSION; }

psph_status psph_device_check(int* device_count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  if (device_count) *device_count = n;
  if (n < 1) return PSPH_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) return PSPH_ERR_NO_DEVICE;
  if (!(prop.major == 10 && prop.minor == 3)) return PSPH_ERR_NO_DEVICE;  // built for sm_103a only
  return PSPH_OK;
}

psph_status psph_create(const psph_config* cfg, psph_ctx** out) { return create_impl(cfg, 1, out); }

void psph_destroy(psph_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  output_writer_destroy(c->out);  // queued snapshots are written first
  free_all(c);
  for (int i = 0; i <= kNumPhases; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* psph_last_error(const psph_ctx* c) { return c ? c->err.c_str() : "null context"; }

psph_status psph_set_stream(psph_ctx* c, void* s) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  if (s) {
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->stream = (cudaStream_t)s;
    c->own_stream = false;
  }
  return PSPH_OK;
}

psph_status psph_set_grid(psph_ctx* c, const psph_grid* g) {
  if (!c || !g) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_set_grid must come before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "psph_set_grid applies to single-domain contexts");
  c->grids[0] = *g;
  c->grid_set = true;
  return PSPH_OK;
}

psph_status psph_set_integrator(psph_ctx* c, const psph_integrator* it) {
  if (!c || !it) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_set_integrator must come before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "psph_set_integrator applies to single-domain contexts");
  c->integ[0] = *it;
  c->integ_set = true;
  return PSPH_OK;
}

psph_status psph_upload(psph_ctx* c, const psph_particles* p, int initial) {
  if (c && c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "an ensemble context takes psph_batch_upload");
  return upload_impl(c, p, initial);
}

psph_status psph_step(psph_ctx* c, int64_t nsteps, double t_stop, int64_t* steps_done) {
  if (c && c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "an ensemble context takes psph_batch_step");
  return step_impl(c, nsteps, nullptr, t_stop, steps_done);
}

int64_t psph_num_particles(const psph_ctx* c) { return num_particles_impl(const_cast<psph_ctx*>(c), 0); }

psph_status psph_download(psph_ctx* c, psph_particles* out) { return download_impl(c, 0, out); }

psph_status psph_original_index(psph_ctx* c, int64_t* out) { return original_index_impl(c, 0, out); }

psph_status psph_get_grid(const psph_ctx* c, psph_grid* g) {
  if (!c || !g) return PSPH_ERR_INVALID_ARGUMENT;
  *g = c->grids[0];
  return PSPH_OK;
}

psph_status psph_get_integrator(const psph_ctx* c, psph_integrator* it) {
  return integrator_impl(const_cast<psph_ctx*>(c), 0, it);
}

psph_status psph_set_step_hooks(psph_ctx* c, psph_hook_fn fn, void* user, int where_mask) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  if (fn && (where_mask & ~(PSPH_HOOK_BEFORE | PSPH_HOOK_AFTER)))
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "where_mask takes PSPH_HOOK_BEFORE and PSPH_HOOK_AFTER");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "step hooks need a single-domain context");
  if (c->in_hook) return set_err(c, PSPH_ERR_STATE, "psph_set_step_hooks inside a hook");
  c->hook_fn = fn;
  c->hook_user = fn ? user : nullptr;
  c->hook_mask = fn ? where_mask : 0;
  return PSPH_OK;
}

psph_status psph_patch(psph_ctx* c, const psph_particles* p) { return patch_impl(c, p); }

psph_status psph_set_flow_profile(psph_ctx* c, int which, psph_flow_fn fn, void* user) {
  if (!c || (which != PSPH_FLOW_IN && which != PSPH_FLOW_OUT)) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->ninst != 1 || c->cfgs[0].in_out_flow <= 0)
    return set_err(c, PSPH_ERR_STATE, "psph_set_flow_profile needs a single domain with in_out_flow set");
  c->flow_fn[which] = fn;
  c->flow_user[which] = fn ? user : nullptr;
  return PSPH_OK;
}

psph_status psph_pairs_export(psph_ctx* c, int which, int64_t* pairs, int64_t cap, int64_t* n_total) {
  if (!c || (which != 0 && which != 1)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export applies to single-domain contexts");
  // cell-sort the current positions (does not change the physical state)
  rearm_kernel<<<1, 256, 0, c->stream>>>(c->d_inst, c->ninst, c->d_sc);
  const DevView v = view_ref(c);
  // this sort runs whatever the step decided, and with a skin the next step
  // sorts and lists again on its own grid
  launch_mark_rebuild(v, true, c->opt.skin > 0.f, c->stream);
  launch_sort(v, c->stream);
  unsigned long long* d_counter = nullptr;
  long long* d_out = nullptr;
  CUDA_TRY(c, cudaMallocAsync((void**)&d_counter, sizeof(unsigned long long), c->stream));
  CUDA_TRY(c, cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), c->stream));
  const long long dcap = (pairs && cap > 0) ? cap : 0;
  CUDA_TRY(c, cudaMallocAsync((void**)&d_out, (size_t)(dcap > 0 ? dcap : 1) * 2 * sizeof(long long), c->stream));
  launch_pairs_export(v, which, d_out, dcap, d_counter, c->stream);
  CUDA_TRY(c, cudaGetLastError());
  unsigned long long total = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&total, d_counter, sizeof total, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (dcap > 0) {
    const long long k = std::min<long long>((long long)total, dcap);
    CUDA_TRY(c, cudaMemcpy(pairs, d_out, (size_t)k * 2 * sizeof(long long), cudaMemcpyDeviceToHost));
  }
  cudaFreeAsync(d_out, c->stream);
  cudaFreeAsync(d_counter, c->stream);
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (n_total) *n_total = (int64_t)total;
  return PSPH_OK;
}

psph_status psph_enable_timing(psph_ctx* c, int enable) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  c->timing = enable != 0;
  return PSPH_OK;
}

psph_status psph_phase_times(const psph_ctx* c, double* ms, int cap, int* n_phases) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  for (int e = 0; e < kNumPhases && e < cap; ++e) ms[e] = c->phase_ms[e];
  if (n_phases) *n_phases = kNumPhases;
  return PSPH_OK;
}

int64_t psph_last_launch_count(const psph_ctx* c) { return c ? c->last_launches : 0; }

int64_t psph_list_rebuilds(psph_ctx* c) {
  if (!c || !c->uploaded || sync_scalars(c)) return -1;
  return (int64_t)c->h_sc->rebuilds;
}

psph_status psph_step_timed(psph_ctx* c, int64_t nsteps, double* device_ms, int64_t* steps_done) {
  if (!c || !device_ms) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_step_timed before psph_upload");
  const bool was = c->timing;
  c->timing = false;
  cudaEvent_t e0, e1;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  // make sure the graph exists before the timed region
  psph_status st = build_graph(c);
  if (st) return st;
  std::vector<int64_t> done(c->ninst, 0);
  CUDA_TRY(c, cudaEventRecord(e0, c->stream));
  st = step_impl(c, nsteps, nullptr, 1e300, done.data());
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->timing = was;
  *device_ms = ms;
  if (steps_done) *steps_done = done[0];
  return st;
}

// Neighbour lists with a skin (the FP32C form): the lists hold every pair
// within (1 + skin) of the support and are kept until a particle has moved
// half the skin; the cell sort and the list scan then use cells of at least
// (1 + skin) Cellfac hmax with the reference's bounds (BLPF, TRPR), so that
// the 3x3(x3) block covers the wider reach. The pair set each step evaluates
// is the same; the summation order follows the kept lists.
psph_status apply_skin(psph_ctx* c, float skin) {
  if (skin > 0.f) {
    if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "a list skin is set after psph_upload");
    if (!c->opt.fp32) return set_err(c, PSPH_ERR_UNSUPPORTED, "list skins apply to the FP32C form (PSPH_FP32C)");
    if (c->opt.any_periodic) return set_err(c, PSPH_ERR_UNSUPPORTED, "list skins apply to domains without a periodic axis");
    for (const PClass& C : c->classes)
      if (C.material == 2)
        return set_err(c, PSPH_ERR_UNSUPPORTED, "list skins apply to fluid and soil domains (Material 2 present)");
    for (const GridDev& g : c->gdevs)
      for (int d = 0; d < 3; ++d)
        if (g.nc[d] > 1023)
          return set_err(c, PSPH_ERR_UNSUPPORTED, "list skins need at most 1023 reference cells per axis (%d)", g.nc[d]);
  }
  std::vector<GridDev> gd(c->gdevs);
  long long base = 0;
  float disp2 = 0.f;
  for (size_t q = 0; q < gd.size(); ++q) {
    GridDev& g = gd[q];
    if (skin > 0.f) {
      const double reach = g.cellfac * g.hmax * (1.0 + (double)skin);
      for (int d = 0; d < 3; ++d) {
        if (g.cell_size[d] <= 0.0) continue;  // an axis beyond the dimension: one cell
        const double L = g.trpr[d] - g.blpf[d];
        const int cn = std::max(1, (int)std::floor(L / reach));
        g.nc[d] = g.cn_ref[d] = cn;
        g.cell_size[d] = L / cn;
        g.inv_cell_size32[d] = (float)(1.0 / g.cell_size[d]);
        g.cell_size32[d] = (float)g.cell_size[d];
      }
      const double half = 0.5 * (double)skin * g.cellfac * g.hmax;
      g.skin_disp2 = (float)(half * half);
      disp2 = (q == 0) ? g.skin_disp2 : std::min(disp2, g.skin_disp2);
    }
    g.ncells = g.nc[0] * g.nc[1] * g.nc[2];
    g.cell_base = (int)base;
    base += g.ncells;
  }
  if (c->uploaded) {  // after the context's own work (its stream), before its next launch
    CUDA_TRY(c, cudaMemcpyAsync(c->d_grids, gd.data(), gd.size() * sizeof(GridDev), cudaMemcpyHostToDevice,
                                c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  c->total_cells = (int)base;
  c->opt.skin = skin;
  c->opt.skin_disp2 = disp2;
  return PSPH_OK;
}

psph_status psph_get_tuning(const psph_ctx* c, psph_tuning* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  out->pair_block = c->opt.pair_block;
  out->cell_split = c->opt.xsub;
  out->nlist_stage = c->opt.nlist_stage;
  out->skin_permille = (int32_t)std::lround(c->opt.skin * 1000.0);
  out->ms_per_step = c->tuned_ms;
  return PSPH_OK;
}

psph_status psph_set_tuning(psph_ctx* c, const psph_tuning* t) {
  if (!c || !t) return PSPH_ERR_INVALID_ARGUMENT;
  if (t->pair_block != 64 && t->pair_block != 128 && t->pair_block != 256)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "pair_block must be 64, 128 or 256 (got %d)", t->pair_block);
  if (t->cell_split != 1 && t->cell_split != 2 && t->cell_split != kMaxXsub)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "cell_split must be 1, 2 or 4 (got %d)", t->cell_split);
  if (t->nlist_stage != 0 && t->nlist_stage != 2048 && t->nlist_stage != 3072 && t->nlist_stage != kMaxStage)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "nlist_stage must be 0, 2048, 3072 or 4096 (got %d)",
                   t->nlist_stage);
  if (t->skin_permille < 0 || t->skin_permille > kMaxSkinPermille)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "skin_permille must lie in [0, %d] (got %d)", kMaxSkinPermille,
                   t->skin_permille);
  const float skin = (float)(t->skin_permille / 1000.0);
  if (c->opt.pair_block != t->pair_block || c->opt.xsub != t->cell_split || c->opt.nlist_stage != t->nlist_stage ||
      c->opt.skin != skin) {
    if (c->opt.skin != skin) {
      psph_status st = apply_skin(c, skin);
      if (st) return st;
    }
    c->opt.pair_block = t->pair_block;
    c->opt.xsub = t->cell_split;
    c->opt.nlist_stage = t->nlist_stage;
    // lists kept with a skin follow the sort's layout: the next step lists again
    if (c->uploaded && c->opt.skin > 0.f) launch_mark_rebuild(view(c), false, true, c->stream);
    if (c->graph) {  // launch parameters change: capture the step again
      cudaGraphExecDestroy(c->graph);
      c->graph = nullptr;
    }
  }
  return PSPH_OK;
}

psph_status psph_autotune(psph_ctx* c, int64_t steps_per_trial, psph_tuning* chosen) {
  if (!c || steps_per_trial < 1) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_autotune before psph_upload");
  std::vector<psph_tuning> cands;
  for (int split : {1, 2, kMaxXsub}) {
    // the pair block only matters for the FP32C pair kernels
    for (int block : {64, 128, 256}) {
      if (!c->opt.fp32 && block != 128) continue;
      psph_tuning t{};
      t.pair_block = block;
      t.cell_split = split;
      cands.push_back(t);
    }
  }
  for (psph_tuning& t : cands) t.nlist_stage = c->opt.nlist_stage;
  psph_tuning best{};
  double best_ms = 1e300;
  bool ended = false;
  auto trial = [&](const psph_tuning& t, int64_t steps) -> psph_status {
    psph_status st = psph_set_tuning(c, &t);
    if (st) return st;
    double ms = 0.0;
    int64_t done = 0;
    if ((st = psph_step_timed(c, 1, &ms, &done))) return st;  // capture + first launch, untimed
    if ((st = psph_step_timed(c, steps, &ms, &done))) return st;
    if (done < steps) {  // the run ended; keep what was measured
      ended = true;
      return PSPH_OK;
    }
    const double per = ms / (double)done;
    if (per < best_ms) {
      best_ms = per;
      best = t;
    }
    return PSPH_OK;
  };
  for (const psph_tuning& t : cands) {
    if (psph_status st = trial(t, steps_per_trial)) return st;
    if (ended) break;
  }
  if (best_ms == 1e300) best = cands.front();
  // then the staging depth of the neighbour search, where it applies
  if (!ended && c->opt.uniform_h && !c->opt.any_periodic_x) {
    const psph_tuning base = best;
    for (int stage : {0, 2048, 3072, kMaxStage}) {
      if (stage == base.nlist_stage) continue;
      psph_tuning t = base;
      t.nlist_stage = stage;
      if (psph_status st = trial(t, steps_per_trial)) return st;
      if (ended) break;
    }
  }
  // then list skins (FP32C): each trial runs long enough for several rebuilds
  // to be in its average
  bool skins = !ended && c->opt.fp32 && !c->opt.any_periodic;
  for (const PClass& C : c->classes) skins = skins && C.material != 2;
  for (const GridDev& g : c->gdevs) skins = skins && g.nc[0] <= 1023 && g.nc[1] <= 1023 && g.nc[2] <= 1023;
  if (skins) {
    const psph_tuning base = best;
    for (int permille : {50, 100, kMaxSkinPermille}) {
      psph_tuning t = base;
      t.skin_permille = permille;
      if (psph_status st = trial(t, std::max<int64_t>(8 * steps_per_trial, 24))) return st;
      if (ended) break;
    }
  }
  psph_status st = psph_set_tuning(c, &best);
  if (st) return st;
  c->tuned_ms = best_ms < 1e300 ? best_ms : 0.0;
  best.ms_per_step = c->tuned_ms;
  if (chosen) *chosen = best;
  return PSPH_OK;
}

psph_status psph_pair_count(psph_ctx* c, uint64_t* pairs) {
  if (!c || !pairs) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) {
    *pairs = 0;
    return PSPH_OK;
  }
  psph_status st = sync_scalars(c);
  if (st) return st;
  *pairs = c->h_sc->pairs_x2 / 2;
  return PSPH_OK;
}

// ---- learned closure -----------------------------------------------------------

psph_status psph_closure_attach(psph_ctx* c, const psph_mlp* mlp, double dx) {
  if (!c || !mlp || !(dx > 0.0)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_closure_attach before psph_upload");
  const MlpImage* img = nullptr;
  psph_status st = psph_mlp_image(mlp, &img);
  if (st) return set_err(c, st, "closure network: %s", psph_mlp_last_error(mlp));
  const size_t N = (size_t)c->ncap;
  if (!c->d_mlp) {
    if ((st = dalloc(c, &c->d_mlp, 1)) || (st = dalloc(c, &c->S.cvort, N)) || (st = dalloc(c, &c->S.cnnb, N)) ||
        (!c->S.cshear && (st = dalloc(c, &c->S.cshear, N))) || (st = dalloc(c, &c->S.cr3, N)) ||
        (st = dalloc(c, &c->S.cfeat, 6 * N)) || (st = dalloc(c, &c->S.nut, N)))
      return st;
  }
  CUDA_TRY(c, cudaMemcpy(c->d_mlp, img, sizeof(MlpImage), cudaMemcpyDeviceToDevice));
  c->opt.closure = 1;
  c->opt.closure_dx = dx;
  {  // the h/dx feature per class, as the FP64 form rounds it
    std::vector<PClass32> c32(c->classes.size());
    CUDA_TRY(c, cudaMemcpy(c32.data(), c->d_cls32, c32.size() * sizeof(PClass32), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < c32.size(); ++q) c32[q].h_over_dx = (float)(c->classes[q].h / dx);
    CUDA_TRY(c, cudaMemcpy(c->d_cls32, c32.data(), c32.size() * sizeof(PClass32), cudaMemcpyHostToDevice));
  }
  if ((st = sync_scalars(c))) return st;
  c->h_sc->closure_eval = 0;
  c->h_sc->closure_fallback = 0;
  CUDA_TRY(c, cudaMemcpy(c->d_sc, c->h_sc, sizeof(StepScalars), cudaMemcpyHostToDevice));
  if (c->graph) {  // the step sequence changes: capture it again
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return PSPH_OK;
}

psph_status psph_closure_stats(psph_ctx* c, uint64_t* evaluated, uint64_t* fallbacks) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_closure_stats before psph_upload");
  psph_status st = sync_scalars(c);
  if (st) return st;
  if (evaluated) *evaluated = c->h_sc->closure_eval;
  if (fallbacks) *fallbacks = c->h_sc->closure_fallback;
  return PSPH_OK;
}

psph_status psph_closure_features(psph_ctx* c, float* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->opt.closure) return set_err(c, PSPH_ERR_STATE, "no closure attached");
  std::vector<std::pair<int, int>> order;
  psph_status st = alive_of(c, 0, order, nullptr);
  if (st) return st;
  const size_t n = (size_t)c->h_sc->n;
  std::vector<float> f(6 * n);
  CUDA_TRY(c, cudaMemcpy(f.data(), c->S.cfeat, 6 * n * sizeof(float), cudaMemcpyDeviceToHost));
  for (size_t r = 0; r < order.size(); ++r)
    for (int k = 0; k < 6; ++k) out[6 * r + k] = f[6 * (size_t)order[r].second + k];
  return PSPH_OK;
}

// ---- ensembles ---------------------------------------------------------------

psph_status psph_batch_create(const psph_config* cfgs, int ninst, psph_ctx** out) {
  return create_impl(cfgs, ninst, out);
}

int psph_batch_size(const psph_ctx* c) { return c ? c->ninst : 0; }

psph_status psph_batch_upload(psph_ctx* c, const psph_particles* parts, int initial) {
  return upload_impl(c, parts, initial);
}

psph_status psph_batch_step(psph_ctx* c, int64_t nsteps, const double* t_stop, int64_t* steps_done) {
  return step_impl(c, nsteps, t_stop, 1e300, steps_done);
}

int64_t psph_batch_num_particles(const psph_ctx* c, int inst) {
  return num_particles_impl(const_cast<psph_ctx*>(c), inst);
}

psph_status psph_batch_download(psph_ctx* c, int inst, psph_particles* out) { return download_impl(c, inst, out); }

psph_status psph_batch_original_index(psph_ctx* c, int inst, int64_t* out) {
  return original_index_impl(c, inst, out);
}

psph_status psph_batch_get_grid(const psph_ctx* c, int inst, psph_grid* g) {
  if (!c || !g || inst < 0 || inst >= c->ninst) return PSPH_ERR_INVALID_ARGUMENT;
  *g = c->grids[inst];
  return PSPH_OK;
}

psph_status psph_batch_get_integrator(const psph_ctx* c, int inst, psph_integrator* it) {
  return integrator_impl(const_cast<psph_ctx*>(c), inst, it);
}

}  // extern "C"

// ---- snapshot output -------------------------------------------------------------

namespace {
psph_status output_prepare(psph_ctx* c, const char* key, const char* const names[3]) {
  if (!c || !key || !*key) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "snapshot output before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "snapshot output applies to single-domain contexts");
  if (!c->out) c->out = output_writer_create();
  c->out_key = key;
  for (int k = 0; k < 3; ++k)
    c->out_names[k] = (names && names[k] && *names[k]) ? names[k] : ("Property" + std::to_string(k + 1));
  return PSPH_OK;
}
}  // namespace

psph_status psph_output_request(psph_ctx* c, const char* file_key, const char* const names[3]) {
  psph_status st = output_prepare(c, file_key, names);
  if (st) return st;
  c->out_requested = true;
  return PSPH_OK;
}

psph_status psph_output_write(psph_ctx* c, const char* file_key, const char* const names[3], const double* prop1,
                              const double* prop2, const double* prop3) {
  psph_status st = output_prepare(c, file_key, names);
  if (st) return st;
  std::string e;
  const int64_t m = num_particles_impl(c, 0);
  std::vector<double> props;
  if (prop1 || prop2 || prop3) {
    props.assign(3 * (size_t)m, 0.0);
    for (int k = 0; k < 3; ++k) {
      const double* p = k == 0 ? prop1 : (k == 1 ? prop2 : prop3);
      if (p) std::copy(p, p + m, props.begin() + (size_t)k * m);
    }
  }
  // (an in/out-flow domain's appended particles take original indices past the upload's)
  const int hi = c->inout ? (int)c->next_orig : (int)c->inst_off[1];
  if (!output_gather(c->out, view(c), 0, hi, c->stream, &e)) return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
  const char* nm[3] = {c->out_names[0].c_str(), c->out_names[1].c_str(), c->out_names[2].c_str()};
  if (!output_commit(c->out, c->out_key.c_str(), nm, props.empty() ? nullptr : props.data(), m, &e) ||
      !output_flush(c->out, &e))
    return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
  return PSPH_OK;
}

psph_status psph_output_flush(psph_ctx* c) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  std::string e;
  if (c->out && !output_flush(c->out, &e)) return set_err(c, PSPH_ERR_CUDA, "%s", e.c_str());
  return PSPH_OK;
}

// ---------------------------------------------------------------------------
// Pair export that allocates nothing.
//
// psph_pairs_export allocates its device counter and output buffer on every
// call. Some callers cannot allocate device memory at the point where they need
// the pairs: code that has handed all device memory to its own pool or to
// another framework's caching allocator (where cudaMalloc fails or fragments),
// and latency-bound loops that must not pay cudaMalloc/cudaFree's device-wide
// synchronisation once running. psph_pairs_export_noalloc serves them: the
// caller passes a device output buffer, the context's cell-sort buffers (made at
// upload) are reused, and the per-particle counts and offsets it needs live in
// one file-scope device array, sized for PSPH_NOALLOC_MAX_PARTICLES particles
// and held by every GPU that loads this library until the process exits.
//
// The array's host-side name is only a stand-in for the device symbol, so the
// address passed to the kernels is taken with cudaGetSymbolAddress, once per
// device (std::call_once, so threads making their first call at the same time
// are safe), by the first call on that device (with that device current); make
// that first call before any stream capture. The address is kept for the
// process: after cudaDeviceReset the module is loaded again and the kept
// address is stale, so the entry point is not for use across a device reset.
// Every call shares the array and overwrites what it needs (nothing in it has
// to start at zero); two calls whose work overlaps on the GPU (different
// streams, or contexts used from several threads) race on it.
//
// The offsets are 32-bit: the pair total is summed in 64 bits first, and a
// total above INT_MAX (PSPH_NOALLOC_MAX_PAIRS) is refused before any pair is
// written.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoallocBlocks = (PSPH_NOALLOC_MAX_PARTICLES + 1023) / 1024 + 2;
constexpr int kNoallocHead = 64;  // ints before the counts: the 64-bit pair total, 256-byte aligned
// total (64-bit) | counts[MAX] | offsets[MAX + 1] | scan block sums
static __device__ __align__(256) int
    g_noalloc_scratch[kNoallocHead + 2 * PSPH_NOALLOC_MAX_PARTICLES + 1 + kNoallocBlocks];

constexpr int kMaxDevices = 64;
std::once_flag g_noalloc_once[kMaxDevices];
int* g_noalloc_addr[kMaxDevices] = {};
cudaError_t g_noalloc_err[kMaxDevices] = {};

psph_status noalloc_scratch(psph_ctx* c, int** out) {
  int dev = -1;
  CUDA_TRY(c, cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_err(c, PSPH_ERR_NO_DEVICE, "device index %d out of range", dev);
  std::call_once(g_noalloc_once[dev], [dev] {
    void* p = nullptr;
    g_noalloc_err[dev] = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    g_noalloc_addr[dev] = (int*)p;
  });
  if (g_noalloc_err[dev] != cudaSuccess || !g_noalloc_addr[dev])
    return set_err(c, PSPH_ERR_CUDA, "cudaGetSymbolAddress of the static pair-export scratch: %s",
                   cudaGetErrorString(g_noalloc_err[dev]));
  *out = g_noalloc_addr[dev];
  return PSPH_OK;
}

// The pair total in 64 bits (one block, a fixed reduction order).
__global__ void __launch_bounds__(1024) noalloc_total_kernel(const int* __restrict__ counts, int n,
                                                             unsigned long long* total) {
  __shared__ unsigned long long part[32];
  unsigned long long s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += (unsigned)counts[i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += part[k];
    *total = t;
  }
}

}  // namespace

extern "C" psph_status psph_pairs_export_noalloc(psph_ctx* c, int which, int64_t* pairs_device, int64_t cap,
                                                 int64_t* n_total) {
  if (!c || (which != 0 && which != 1) || cap < 0 || (cap > 0 && !pairs_device)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export_noalloc before psph_upload");
  if (c->ninst != 1) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export_noalloc applies to single-domain contexts");
  if (c->ncap > PSPH_NOALLOC_MAX_PARTICLES)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT,
                   "psph_pairs_export_noalloc handles at most %d particles (context holds %d); use psph_pairs_export",
                   PSPH_NOALLOC_MAX_PARTICLES, c->ncap);
  int* scratch = nullptr;
  psph_status st = noalloc_scratch(c, &scratch);
  if (st) return st;
  unsigned long long* d_total = reinterpret_cast<unsigned long long*>(scratch);
  int* counts = scratch + kNoallocHead;
  int* offsets = counts + PSPH_NOALLOC_MAX_PARTICLES;
  int* block_sums = offsets + PSPH_NOALLOC_MAX_PARTICLES + 1;
  cudaStream_t s = c->stream;
  rearm_kernel<<<1, 256, 0, s>>>(c->d_inst, c->ninst, c->d_sc);
  const DevView v = view_ref(c);                       // the reference's cells, also with a skin
  launch_mark_rebuild(v, true, c->opt.skin > 0.f, s);  // this sort runs; a skin's lists follow next step
  launch_sort(v, s);                                   // cell list of the current positions
  launch_pairs_count(v, which, counts, s);             // pairs each sorted particle lists first
  noalloc_total_kernel<<<1, 1024, 0, s>>>(counts, c->ncap, d_total);
  CUDA_TRY(c, cudaGetLastError());
  unsigned long long total = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&total, d_total, sizeof total, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(c, cudaStreamSynchronize(s));
  if (total > (unsigned long long)PSPH_NOALLOC_MAX_PAIRS)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT,
                   "psph_pairs_export_noalloc: %llu pairs exceed its 32-bit offsets (at most %d); use "
                   "psph_pairs_export",
                   total, PSPH_NOALLOC_MAX_PAIRS);
  if (cap > 0 && total > 0) {
    launch_exclusive_scan(counts, offsets, c->ncap, block_sums, s);
    launch_pairs_write(v, which, offsets, (long long*)pairs_device, (long long)cap, s);
    CUDA_TRY(c, cudaGetLastError());
    CUDA_TRY(c, cudaStreamSynchronize(s));
  }
  if (n_total) *n_total = (int64_t)total;
  return PSPH_OK;
}
