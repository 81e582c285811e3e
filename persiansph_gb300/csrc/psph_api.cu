// C ABI of the GB300 hot path (include/psph.h): context, upload/download,
// Solve's set-up on the host (InitialChecks, CellInitiate, TimestepCheck), and
// the per-step launch sequence captured once into a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "psph_device.cuh"

using namespace psph;

struct psph_ctx {
  psph_config cfg{};
  psph_grid grid{};
  bool grid_set = false;
  psph_integrator integ{};
  bool integ_set = false;
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int ncap = 0;
  int n_upload = 0;
  std::vector<PClass> classes;
  Options opt{};
  GridDev gdev{};
  Persist PA{}, PB{};
  Scratch S{};
  PClass* d_cls = nullptr;
  PClass32* d_cls32 = nullptr;
  StepScalars* d_sc = nullptr;
  StepScalars* h_sc = nullptr;  // pinned mirror
  uint8_t* d_alive = nullptr;
  std::vector<void*> allocs;
  cudaGraphExec_t graph = nullptr;
  bool uploaded = false;
  bool timing = false;
  double phase_ms[5] = {0, 0, 0, 0, 0};
  long long last_launches = 0;
  cudaEvent_t ev[6] = {};
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
}

// Particle constructor defaults (Source/Particle.cpp:25-117) for NULL arrays.
double dflt(const double* a, int64_t i, double d) { return a ? a[i] : d; }
int32_t iflt(const int32_t* a, int64_t i, int32_t d) { return a ? a[i] : d; }

double eos_host(int eq, double cs, double p0, double rho, double rho0) {
  switch (eq) {  // Source/Functions.cpp:188-212, same expression order
    case 0: return p0 + (cs * cs) * (rho - rho0);
    case 1: return p0 + (rho0 * cs * cs / 7.0) * (std::pow(rho / rho0, 7.0) - 1);
    default: return (cs * cs) * rho;
  }
}

// CellInitiate (Source/Domain.cpp:549-660).
psph_status cell_initiate(psph_ctx* c, const psph_particles* p, double* mu_max, double* cs_max) {
  psph_grid& g = c->grid;
  const int64_t n = p->n;
  double TRPR[3], BLPF[3];
  for (int d = 0; d < 3; ++d) TRPR[d] = BLPF[d] = p->x[d];
  double hmax = p->h[0];
  double rhomax = p->density[0];
  *mu_max = 0.0;
  *cs_max = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) {
      const double xd = p->x[3 * i + d];
      if (xd > TRPR[d]) TRPR[d] = xd;
      if (xd < BLPF[d]) BLPF[d] = xd;
    }
    if (p->h[i] > hmax) hmax = p->h[i];
    if (p->density[i] > rhomax) rhomax = p->density[i];
    const double mu = dflt(p->mu, i, 0.0), cs = dflt(p->cs, i, 0.0);
    if (mu > *mu_max) *mu_max = mu;
    if (cs > *cs_max) *cs_max = cs;
  }
  const psph_config& cf = c->cfg;
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
  v.g = c->gdev;
  v.o = c->opt;
  v.PA = c->PA;
  v.PB = c->PB;
  v.S = c->S;
  v.cls = c->d_cls;
  v.cls32 = c->d_cls32;
  v.sc = c->d_sc;
  v.alive = c->d_alive;
  v.ncap = c->ncap;
  v.nclasses = (int)c->classes.size();
  return v;
}

// One step of Solve's loop body (Source/Domain.cpp:1764-1792) as launches.
void enqueue_step(psph_ctx* c) {
  const DevView v = view(c);
  cudaStream_t st = c->stream;
  launch_begin(v, st);
  record_phase(c, 0);
  launch_sort(v, st);
  launch_nlist(v, st);
  record_phase(c, 1);
  if (v.o.fp32) launch_prepare32(v, st);
  else launch_prepare(v, st);
  record_phase(c, 2);
  if (v.o.fp32) launch_forces32(v, st);
  else launch_forces(v, st);
  record_phase(c, 3);
  launch_dt(v, st);
  record_phase(c, 4);
  launch_update(v, st);
  launch_end(v, st);
  record_phase(c, 5);
}

__global__ void arm_kernel(StepScalars* sc, double t_stop) {
  sc->t_stop = t_stop;
  sc->stop = 0;
  sc->status = 0;
}

psph_status sync_scalars(psph_ctx* c) {
  CUDA_TRY(c, cudaMemcpyAsync(c->h_sc, c->d_sc, sizeof(StepScalars), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
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

psph_status psph_create(const psph_config* cfg, psph_ctx** out) {
  if (!cfg || !out) return PSPH_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  psph_ctx* c = new psph_ctx();
  c->cfg = *cfg;
  *out = c;
  const psph_config& k = *cfg;
  if (k.dimension != 2 && k.dimension != 3)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Please correct the dimension (2=>2D or 3=>3D) and run again");
  if (k.kernel_type < 0 || k.kernel_type > 2)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Kernel Type No is out of range");
  if (k.vis_eq < 0 || k.vis_eq > 3) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Viscosity Equation No is out of range");
  if (k.gradient_type < 0 || k.gradient_type > 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Gradient type out of range");
  if (k.scheme != PSPH_MVERLET && k.scheme != PSPH_LEAPFROG)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Scheme must be 0 (Modified Verlet) or 1 (Leapfrog)");
  if (k.swi_type != 0) return set_err(c, PSPH_ERR_UNSUPPORTED, "soil-water interaction (SWIType) is outside this build");
  if (k.precision != PSPH_FP64 && k.precision != PSPH_FP32C)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "precision must be PSPH_FP64 or PSPH_FP32C");
  if (k.dimension == 2 && k.periodic[2]) return set_err(c, PSPH_ERR_UNSUPPORTED, "periodic z in 2D");
  for (int e = 0; e < 8; ++e)
    if (k.reserved[e]) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "reserved fields must be zero");
  int dev = 0;
  if (psph_device_check(&dev) != PSPH_OK) return set_err(c, PSPH_ERR_NO_DEVICE, "no sm_103 CUDA device available");
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  c->own_stream = true;
  for (int i = 0; i < 6; ++i) cudaEventCreate(&c->ev[i]);
  c->integ.time = k.time;
  c->integ.deltat = c->integ.deltatint = c->integ.deltatmin = k.dt;
  c->integ.first_step = 1;
  return PSPH_OK;
}

void psph_destroy(psph_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_all(c);
  for (int i = 0; i < 6; ++i)
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
  c->grid = *g;
  c->grid_set = true;
  return PSPH_OK;
}

psph_status psph_set_integrator(psph_ctx* c, const psph_integrator* it) {
  if (!c || !it) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_set_integrator must come before psph_upload");
  c->integ = *it;
  c->integ_set = true;
  return PSPH_OK;
}

psph_status psph_upload(psph_ctx* c, const psph_particles* p, int initial) {
  if (!c || !p) return PSPH_ERR_INVALID_ARGUMENT;
  if (c->uploaded) return set_err(c, PSPH_ERR_STATE, "particles already uploaded to this context");
  if (!c->stream) return set_err(c, PSPH_ERR_STATE, "context not created");
  const int64_t n = p->n;
  if (n < 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "no particles");
  if (n > (1LL << 30)) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "too many particles");
  if (!p->x || !p->h || !p->density || !p->mass)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "x, h, density and mass are required");
  const psph_config& k = c->cfg;
  const bool lf = (k.scheme == PSPH_LEAPFROG);

  // ---- particle classes ---------------------------------------------------
  std::vector<int> cls(n);
  std::unordered_map<std::string, int, ClassKeyHash> index;
  bool dyn_mu = false;
  for (int64_t i = 0; i < n; ++i)
    if (dflt(p->t0, i, 0.0) > 0.0 || iflt(p->les, i, 0)) dyn_mu = true;
  std::vector<double> pressure(n);
  int material0 = -1;
  for (int64_t i = 0; i < n; ++i) {
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
    if (C.material < 1 || C.material > 3)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Material Type No is out of range (particle %lld)", (long long)i);
    if (C.pres_eq < 0 || C.pres_eq > 2)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Please correct Pressure Equation No (particle %lld)", (long long)i);
    if (C.material == 2 && C.fail > 1) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Undefined failure criteria for solids");
    if (C.material == 3 && C.fail > 3) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Failure Type No is out of range");
    if (C.material == 1 && C.t0 > 0.0 && C.vis_m > 1)
      return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "Non-Newtonian Viscosity Type No is out of range");
    if (material0 < 0) material0 = C.material;
    if (C.material != material0)
      return set_err(c, PSPH_ERR_UNSUPPORTED,
                     "particles of different materials interact through CalcForce12/13 (FSI, seepage), outside this build");
    std::string key((const char*)&C, sizeof C);
    auto it = index.find(key);
    int id;
    if (it == index.end()) {
      id = (int)c->classes.size();
      if (id >= 65535) return set_err(c, PSPH_ERR_UNSUPPORTED, "more than 65535 distinct particle parameter sets");
      index.emplace(key, id);
      c->classes.push_back(C);
    } else {
      id = it->second;
    }
    cls[i] = id;
    // InitialChecks: initial pressure from the EOS for fluids and solids (Source/Domain.cpp:1675-1677)
    const double p_in = dflt(p->pressure, i, 0.0);
    pressure[i] = (initial && C.material < 3) ? eos_host(C.pres_eq, C.cs, C.p0, p->density[i], C.rho0) : p_in;
  }

  // ---- grid (CellInitiate) and TimestepCheck --------------------------------
  if (!c->grid_set) {
    double mu_max, cs_max;
    psph_status st = cell_initiate(c, p, &mu_max, &cs_max);
    if (st) return st;
    if (initial) {  // TimestepCheck (Source/Domain.cpp:1721-1733)
      const double t1 = 0.25 * c->grid.hmax / (cs_max);
      const double t2 = (mu_max > 0.0) ? 0.125 * c->grid.hmax * c->grid.hmax * c->grid.rhomax / mu_max : 1000000.0;
      if (c->integ.deltatint > std::min(t1, t2))
        return set_err(c, PSPH_ERR_CFL, "Please decrease the time step to the allowable range (CFL limit %g s)",
                       std::min(t1, t2));
    }
  }
  GridDev& gd = c->gdev;
  for (int d = 0; d < 3; ++d) {
    gd.blpf[d] = c->grid.blpf[d];
    gd.trpr[d] = c->grid.trpr[d];
    gd.cell_size[d] = c->grid.cell_size[d];
    gd.dom_size[d] = c->grid.dom_size[d];
    gd.periodic[d] = k.periodic[d] ? 1 : 0;
    gd.cn_ref[d] = c->grid.cell_no[d];
    gd.nc[d] = k.periodic[d] ? c->grid.cell_no[d] - 2 : c->grid.cell_no[d];
    if (k.periodic[d] && gd.nc[d] < 3)
      return set_err(c, PSPH_ERR_UNSUPPORTED, "periodic axis %d spans fewer than 3 cells", d);
  }
  gd.hmax = c->grid.hmax;
  gd.cellfac = (k.kernel_type == PSPH_QUINTIC_SPLINE) ? 3.0 : 2.0;
  c->grid.cellfac = gd.cellfac;
  const long long ncells = (long long)gd.nc[0] * gd.nc[1] * gd.nc[2];
  if (ncells > (1LL << 30)) return set_err(c, PSPH_ERR_UNSUPPORTED, "grid has more than 2^30 cells");
  gd.ncells = (int)ncells;

  // ---- options ---------------------------------------------------------------
  Options& o = c->opt;
  o.dim = k.dimension;
  o.kt = k.kernel_type;
  o.vis_eq = k.vis_eq;
  o.grad_type = k.gradient_type;
  o.scheme = k.scheme;
  o.wallp_physical = (k.wall_pressure_mode == PSPH_WALLP_PHYSICAL);
  o.has_solid = (material0 > 1);
  o.fp32 = (k.precision == PSPH_FP32C);
  if (o.fp32 && o.has_solid)
    return set_err(c, PSPH_ERR_UNSUPPORTED, "the FP32C form covers fluids (Material 1); use PSPH_FP64 for solids and soil");
  if (n >= (1LL << 26)) return set_err(c, PSPH_ERR_UNSUPPORTED, "this build handles fewer than 2^26 particles");
  o.soil_pairs = (material0 == 3);
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
  o.any_av = o.any_ti = o.need_sr = o.any_shepard = 0;
  for (size_t q = 0; q < c->classes.size(); ++q) {
    const PClass& C = c->classes[q];
    if (C.h != c->classes[0].h) o.uniform_h = 0;
    if (C.alpha != 0.0 || C.beta != 0.0) o.any_av = 1;
    if (C.ti > 0.0) o.any_ti = 1;
    if (C.material == 1 && (C.t0 > 0.0 || C.les)) o.need_sr = 1;
    if (C.shepard) o.any_shepard = 1;
    if (C.is_free) {
      if (o.eos_cls < 0) o.eos_cls = (int)q;
      else {
        const PClass& E = c->classes[o.eos_cls];
        if (E.pres_eq != C.pres_eq || E.cs != C.cs || E.p0 != C.p0 || E.rho0 != C.rho0) o.uniform_eos = 0;
      }
    }
  }
  if (o.eos_cls < 0) o.eos_cls = 0;
  o.uniform_mu = !dyn_mu;
  o.mu_u = 0.0;
  {
    bool first = true;
    for (const PClass& C : c->classes)
      if (C.is_free) {
        if (first) { o.mu_u = C.mu0; first = false; }
        else if (C.mu0 != o.mu_u) o.uniform_mu = 0;
      }
    // zero viscosity keeps the reference's 0/0 harmonic mean (Source/Interaction.cpp:103)
    if (!(o.mu_u > 0.0)) o.uniform_mu = 0;
  }
  o.inv_h = 1.0 / c->classes[0].h;
  o.nclasses = (int)c->classes.size();

  // ---- device buffers ----------------------------------------------------------
  c->ncap = (int)n;
  c->n_upload = (int)n;
  const size_t N = (size_t)n;
  psph_status st = PSPH_OK;
  for (Persist* P : {&c->PA, &c->PB}) {
    if ((st = dalloc(c, &P->X4, N)) || (st = dalloc(c, &P->V4, N)) || (st = dalloc(c, &P->H4, N)) ||
        (st = dalloc(c, &P->cls, N)) || (st = dalloc(c, &P->orig, N)))
      return st;
    if (lf && (st = dalloc(c, &P->H4b, N))) return st;
    if (dyn_mu && (st = dalloc(c, &P->mu, N))) return st;
    if (o.has_solid) {
      if ((st = dalloc(c, &P->sigma, 9 * N)) || (st = dalloc(c, &P->sigma_h, 9 * N)) ||
          (st = dalloc(c, &P->strain, 9 * N)) || (st = dalloc(c, &P->strain_h, 9 * N)) ||
          (st = dalloc(c, &P->shear, 9 * N)) || (st = dalloc(c, &P->shear_h, 9 * N)) ||
          (st = dalloc(c, &P->tir, 9 * N)))
        return st;
    }
  }
  Scratch& S = c->S;
  const size_t NC = (size_t)ncells;
  const int nb_forces = forces_blocks((int)n);
  if ((st = dalloc(c, &S.key, N)) || (st = dalloc(c, &S.count, NC + 2)) || (st = dalloc(c, &S.start, NC + 3)) ||
      (st = dalloc(c, &S.tmp_perm, N)) || (st = dalloc(c, &S.perm, N)) || (st = dalloc(c, &S.cellid, N)) ||
      (st = dalloc(c, &S.block_sums, (NC + 2 + 1023) / 1024 + 1)) || (st = dalloc(c, &S.blockmin, (size_t)nb_forces)) ||
      (st = dalloc(c, &S.OFF32, N)) || (st = dalloc(c, &S.D4, N)) || (st = dalloc(c, &S.nl_count, N)) ||
      (st = dalloc(c, &S.A4, N)) || (st = dalloc(c, &S.zwab, N)) || (st = dalloc(c, &S.sumden, N)) ||
      (st = dalloc(c, &S.sumkernel, N)) || (st = dalloc(c, &S.nsv4, N)) || (st = dalloc(c, &S.vxsph4, N)) ||
      (st = dalloc(c, &S.shear_rate, N)) || (st = dalloc(c, &S.sbar, N)))
    return st;
  if (o.need_sr || o.has_solid)
    if ((st = dalloc(c, &S.strain_rate, 9 * N))) return st;
  if (o.fp32)
    if ((st = dalloc(c, &S.V32, N)) || (st = dalloc(c, &S.D32, N))) return st;
  // neighbour lists: 3D supports hold ~80 (h = 1.3 dx) particles, 2D ~20-44;
  // a particle with more falls back to scanning its cells
  o.nl_cap = (k.dimension == 3) ? 128 : 64;
  if ((st = dalloc(c, &S.nl, (size_t)o.nl_cap * N))) return st;
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
      F.pad = 0;
    }
    if ((st = dalloc(c, &c->d_cls32, c32.size()))) return st;
    CUDA_TRY(c, cudaMemcpy(c->d_cls32, c32.data(), c32.size() * sizeof(PClass32), cudaMemcpyHostToDevice));
  }
  if (o.has_solid) {
    if ((st = dalloc(c, &S.rotation_rate, 9 * N)) || (st = dalloc(c, &S.sigma_o, 9 * N)) ||
        (st = dalloc(c, &S.strain_o, 9 * N)) || (st = dalloc(c, &S.shear_o, 9 * N)))
      return st;
  }
  if ((st = dalloc(c, &c->d_cls, c->classes.size())) || (st = dalloc(c, &c->d_sc, 1)) || (st = dalloc(c, &c->d_alive, N)))
    return st;
  CUDA_TRY(c, cudaMallocHost(&c->h_sc, sizeof(StepScalars)));

  // ---- pack and copy --------------------------------------------------------------
  {
    std::vector<double4_32a> X(N), V(N), H(N), Hb(lf ? N : 0);
    std::vector<int> orig(N);
    for (int64_t i = 0; i < n; ++i) {
      const double* x = p->x + 3 * i;
      const bool two_d = (k.dimension == 2);
      const double vx = dflt(p->v, 3 * i, 0.0), vy = dflt(p->v, 3 * i + 1, 0.0),
                   vz = two_d ? 0.0 : dflt(p->v, 3 * i + 2, 0.0);
      X[i] = make_double4_32a(x[0], x[1], x[2], p->density[i]);
      V[i] = make_double4_32a(vx, vy, vz, pressure[i]);
      if (lf) {
        H[i] = make_double4_32a(dflt(p->va, 3 * i, 0.0), dflt(p->va, 3 * i + 1, 0.0), dflt(p->va, 3 * i + 2, 0.0),
                            dflt(p->densitya, i, 0.0));
        Hb[i] = make_double4_32a(dflt(p->vb, 3 * i, 0.0), dflt(p->vb, 3 * i + 1, 0.0), dflt(p->vb, 3 * i + 2, 0.0),
                             dflt(p->densityb, i, 0.0));
      } else {
        H[i] = make_double4_32a(dflt(p->vb, 3 * i, 0.0), dflt(p->vb, 3 * i + 1, 0.0), dflt(p->vb, 3 * i + 2, 0.0),
                            dflt(p->densityb, i, 0.0));
      }
      orig[i] = (int)i;
    }
    CUDA_TRY(c, cudaMemcpy(c->PA.X4, X.data(), N * sizeof(double4_32a), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->PA.V4, V.data(), N * sizeof(double4_32a), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->PA.H4, H.data(), N * sizeof(double4_32a), cudaMemcpyHostToDevice));
    if (lf) CUDA_TRY(c, cudaMemcpy(c->PA.H4b, Hb.data(), N * sizeof(double4_32a), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->PA.cls, cls.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->PA.orig, orig.data(), N * sizeof(int), cudaMemcpyHostToDevice));
    if (dyn_mu) {
      std::vector<double> mu(N);
      for (int64_t i = 0; i < n; ++i) mu[i] = dflt(p->mu, i, 0.0);
      CUDA_TRY(c, cudaMemcpy(c->PA.mu, mu.data(), N * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (o.has_solid) {
      const double* srcs[7] = {p->sigma, lf ? p->sigmaa : p->sigmab, p->strain, lf ? p->straina : p->strainb,
                               p->shear_stress, lf ? p->shear_stressa : p->shear_stressb, p->tir};
      double* dsts[7] = {c->PA.sigma, c->PA.sigma_h, c->PA.strain, c->PA.strain_h, c->PA.shear, c->PA.shear_h, c->PA.tir};
      for (int a = 0; a < 7; ++a)
        if (srcs[a]) CUDA_TRY(c, cudaMemcpy(dsts[a], srcs[a], 9 * N * sizeof(double), cudaMemcpyHostToDevice));
    }
    std::vector<uint8_t> alive(N, 1);
    CUDA_TRY(c, cudaMemcpy(c->d_alive, alive.data(), N, cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_cls, c->classes.data(), c->classes.size() * sizeof(PClass), cudaMemcpyHostToDevice));
    StepScalars sc;
    std::memset(&sc, 0, sizeof sc);
    sc.time = c->integ.time;
    sc.deltat = c->integ.deltat;
    sc.deltatint = c->integ.deltatint;
    sc.deltatmin = c->integ.deltatmin;
    sc.steps = c->integ.steps;
    sc.first_step = c->integ.first_step;
    sc.ct = c->integ.ct;
    sc.shepard_counter = c->integ.shepard_counter;
    sc.n = (int)n;
    sc.n_total = (int)n;
    sc.buf = 0;
    sc.t_stop = 1e300;
    CUDA_TRY(c, cudaMemcpy(c->d_sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
  }
  c->uploaded = true;
  return PSPH_OK;
}

psph_status psph_step(psph_ctx* c, int64_t nsteps, double t_stop, int64_t* steps_done) {
  if (!c) return PSPH_ERR_INVALID_ARGUMENT;
  if (steps_done) *steps_done = 0;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_step before psph_upload");
  psph_status st;
  if (nsteps <= 0) {
    if (!c->timing && !c->graph) {
      cudaGraph_t g;
      CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_step(c);
      cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
    return PSPH_OK;
  }
  if ((st = sync_scalars(c))) return st;
  const long long steps0 = c->h_sc->steps;
  arm_kernel<<<1, 1, 0, c->stream>>>(c->d_sc, t_stop);
  CUDA_TRY(c, cudaGetLastError());
  for (int e = 0; e < 5; ++e) c->phase_ms[e] = 0.0;
  long long launched = 0;
  if (c->timing) {
    for (int64_t s = 0; s < nsteps; ++s) {
      enqueue_step(c);
      CUDA_TRY(c, cudaGetLastError());
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      for (int e = 0; e < 5; ++e) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[e], c->ev[e + 1]);
        c->phase_ms[e] += ms;
      }
      launched += launches_per_step(view(c));
      if ((st = sync_scalars(c))) return st;
      if (c->h_sc->stop) break;
    }
  } else {
    if (!c->graph) {
      cudaGraph_t g;
      CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_step(c);
      cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&c->graph, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return set_err(c, PSPH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    }
    int64_t left = nsteps;
    while (left > 0) {
      const int64_t chunk = std::min<int64_t>(left, 256);
      for (int64_t s = 0; s < chunk; ++s) CUDA_TRY(c, cudaGraphLaunch(c->graph, c->stream));
      left -= chunk;
      launched += chunk * launches_per_step(view(c));
      if ((st = sync_scalars(c))) return st;
      if (c->h_sc->stop || c->h_sc->status) break;
    }
  }
  if ((st = sync_scalars(c))) return st;
  const long long done = c->h_sc->steps - steps0;
  if (steps_done) *steps_done = done;
  c->last_launches = launched;
  const uint32_t status = c->h_sc->status;
  if (status & ST_DT_COLLAPSE)
    return set_err(c, PSPH_ERR_DT_COLLAPSE,
                   "Too small time step, please choose a smaller time step initially to make the simulation more stable");
  if (status & ST_OUT_OF_GRID)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "a particle lies more than hmax outside the cell grid");
  if (status & ST_NONFINITE) return set_err(c, PSPH_ERR_NONFINITE, "non-finite acceleration or density rate");
  return PSPH_OK;
}

int64_t psph_num_particles(const psph_ctx* c) {
  if (!c || !c->uploaded) return 0;
  psph_ctx* m = const_cast<psph_ctx*>(c);
  if (sync_scalars(m)) return -1;
  // alive slots: the last update may have flagged leavers that the next sort removes
  std::vector<uint8_t> alive(m->h_sc->n);
  cudaMemcpy(alive.data(), m->d_alive, alive.size(), cudaMemcpyDeviceToHost);
  int64_t k = 0;
  for (uint8_t a : alive) k += a;
  return k;
}

psph_status psph_download(psph_ctx* c, psph_particles* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_download before psph_upload");
  psph_status st;
  if ((st = sync_scalars(c))) return st;
  const StepScalars sc = *c->h_sc;
  const size_t n = (size_t)sc.n;
  const Persist& P = sc.buf ? c->PB : c->PA;
  const Options& o = c->opt;
  const bool lf = (o.scheme == PSPH_LEAPFROG);
  std::vector<uint8_t> alive(n);
  std::vector<int> orig(n), cls(n);
  CUDA_TRY(c, cudaMemcpy(alive.data(), c->d_alive, n, cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(orig.data(), P.orig, n * sizeof(int), cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(cls.data(), P.cls, n * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<std::pair<int, int>> order;
  order.reserve(n);
  for (size_t s = 0; s < n; ++s)
    if (alive[s]) order.emplace_back(orig[s], (int)s);
  std::sort(order.begin(), order.end());
  const int64_t m = (int64_t)order.size();
  if (out->n < m) return set_err(c, PSPH_ERR_INVALID_ARGUMENT, "output holds %lld particles, need %lld", (long long)out->n, (long long)m);
  out->n = m;
  auto fetch4 = [&](const double4_32a* src, std::vector<double4_32a>& dst) -> psph_status {
    dst.resize(n);
    CUDA_TRY(c, cudaMemcpy(dst.data(), src, n * sizeof(double4_32a), cudaMemcpyDeviceToHost));
    return PSPH_OK;
  };
  auto fetch = [&](const double* src, size_t per, std::vector<double>& dst) -> psph_status {
    dst.resize(n * per);
    CUDA_TRY(c, cudaMemcpy(dst.data(), src, n * per * sizeof(double), cudaMemcpyDeviceToHost));
    return PSPH_OK;
  };
  std::vector<double4_32a> b4;
  auto put4 = [&](double* vec3, double* scal, bool xyz) {
    for (int64_t r = 0; r < m; ++r) {
      const double4_32a q = b4[order[r].second];
      if (vec3 && xyz) {
        vec3[3 * r] = q.x;
        vec3[3 * r + 1] = q.y;
        vec3[3 * r + 2] = q.z;
      }
      if (scal) scal[r] = q.w;
    }
  };
  if (out->x || out->density) { if ((st = fetch4(P.X4, b4))) return st; put4(out->x, out->density, true); }
  if (out->v || out->pressure) { if ((st = fetch4(P.V4, b4))) return st; put4(out->v, out->pressure, true); }
  if (lf) {
    if (out->va || out->densitya) { if ((st = fetch4(P.H4, b4))) return st; put4(out->va, out->densitya, true); }
    if (out->vb || out->densityb) { if ((st = fetch4(P.H4b, b4))) return st; put4(out->vb, out->densityb, true); }
  } else {
    if (out->vb || out->densityb) { if ((st = fetch4(P.H4, b4))) return st; put4(out->vb, out->densityb, true); }
  }
  if (out->a || out->ddensity) { if ((st = fetch4(c->S.A4, b4))) return st; put4(out->a, out->ddensity, true); }
  if (out->nsv) { if ((st = fetch4(c->S.nsv4, b4))) return st; put4(out->nsv, nullptr, true); }
  if (out->vxsph) { if ((st = fetch4(c->S.vxsph4, b4))) return st; put4(out->vxsph, nullptr, true); }
  std::vector<double> b;
  auto put = [&](double* dst, size_t per) {
    for (int64_t r = 0; r < m; ++r)
      for (size_t e = 0; e < per; ++e) dst[per * r + e] = b[per * order[r].second + e];
  };
  struct Src { double* out; const double* dev; size_t per; };
  const Src scalars[] = {
      {out->zwab, c->S.zwab, 1}, {out->sumden, c->S.sumden, 1}, {out->sumkernel, c->S.sumkernel, 1},
      {out->shear_rate, c->S.shear_rate, 1}, {out->sbar, c->S.sbar, 1},
      {out->mu, o.dyn_mu ? P.mu : nullptr, 1},
      {out->strain_rate, c->S.strain_rate, 9}, {out->rotation_rate, c->S.rotation_rate, 9},
      {out->sigma, P.sigma, 9}, {out->strain, P.strain, 9}, {out->shear_stress, P.shear, 9}, {out->tir, P.tir, 9},
      {lf ? out->sigmaa : out->sigmab, P.sigma_h, 9}, {lf ? out->sigmab : nullptr, c->S.sigma_o, 9},
      {lf ? out->straina : out->strainb, P.strain_h, 9}, {lf ? out->strainb : nullptr, c->S.strain_o, 9},
      {lf ? out->shear_stressa : out->shear_stressb, P.shear_h, 9}, {lf ? out->shear_stressb : nullptr, c->S.shear_o, 9},
  };
  for (const Src& s : scalars) {
    if (!s.out || !s.dev) continue;
    if ((st = fetch(s.dev, s.per, b))) return st;
    put(s.out, s.per);
  }
  // class constants
  for (int64_t r = 0; r < m; ++r) {
    const PClass& C = c->classes[cls[order[r].second]];
    if (out->id) out->id[r] = C.id;
    if (out->material) out->material[r] = C.material;
    if (out->is_free) out->is_free[r] = C.is_free;
    if (out->no_slip) out->no_slip[r] = C.no_slip;
    if (out->pres_eq) out->pres_eq[r] = C.pres_eq;
    if (out->shepard) out->shepard[r] = C.shepard;
    if (out->les) out->les[r] = C.les;
    if (out->vis_m) out->vis_m[r] = C.vis_m;
    if (out->fail) out->fail[r] = C.fail;
    if (out->mass) out->mass[r] = C.mass;
    if (out->h) out->h[r] = C.h;
    if (out->cs) out->cs[r] = C.cs;
    if (out->p0) out->p0[r] = C.p0;
    if (out->ref_density) out->ref_density[r] = C.rho0;
    if (out->fpmassc) out->fpmassc[r] = C.fpmassc;
    if (out->alpha) out->alpha[r] = C.alpha;
    if (out->beta) out->beta[r] = C.beta;
    if (out->mu && !o.dyn_mu) out->mu[r] = C.mu0;
    if (out->mu_ref) out->mu_ref[r] = C.mu_ref;
    if (out->t0) out->t0[r] = C.t0;
    if (out->bingham_m) out->bingham_m[r] = C.bm;
    if (out->csmag) out->csmag[r] = C.csmag;
    if (out->ti) out->ti[r] = C.ti;
    if (out->tin) out->tin[r] = C.tin;
    if (out->ti_init_dist) out->ti_init_dist[r] = C.tid;
    if (out->g_mod) out->g_mod[r] = C.g_mod;
    if (out->k_mod) out->k_mod[r] = C.k_mod;
    if (out->sigmay) out->sigmay[r] = C.sigmay;
    if (out->cohesion) out->cohesion[r] = C.coh;
    if (out->phi) out->phi[r] = C.phi;
    if (out->psi) out->psi[r] = C.psi;
  }
  return PSPH_OK;
}

psph_status psph_original_index(psph_ctx* c, int64_t* out) {
  if (!c || !out) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_original_index before psph_upload");
  psph_status st;
  if ((st = sync_scalars(c))) return st;
  const StepScalars sc = *c->h_sc;
  const size_t n = (size_t)sc.n;
  const Persist& P = sc.buf ? c->PB : c->PA;
  std::vector<uint8_t> alive(n);
  std::vector<int> orig(n);
  CUDA_TRY(c, cudaMemcpy(alive.data(), c->d_alive, n, cudaMemcpyDeviceToHost));
  CUDA_TRY(c, cudaMemcpy(orig.data(), P.orig, n * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> kept;
  for (size_t s = 0; s < n; ++s)
    if (alive[s]) kept.push_back(orig[s]);
  std::sort(kept.begin(), kept.end());
  for (size_t r = 0; r < kept.size(); ++r) out[r] = kept[r];
  return PSPH_OK;
}

psph_status psph_get_grid(const psph_ctx* c, psph_grid* g) {
  if (!c || !g) return PSPH_ERR_INVALID_ARGUMENT;
  *g = c->grid;
  return PSPH_OK;
}

psph_status psph_get_integrator(const psph_ctx* c, psph_integrator* it) {
  if (!c || !it) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) {
    *it = c->integ;
    return PSPH_OK;
  }
  psph_ctx* m = const_cast<psph_ctx*>(c);
  psph_status st = sync_scalars(m);
  if (st) return st;
  const StepScalars& s = *m->h_sc;
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

psph_status psph_pairs_export(psph_ctx* c, int which, int64_t* pairs, int64_t cap, int64_t* n_total) {
  if (!c || (which != 0 && which != 1)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export before psph_upload");
  // cell-sort the current positions (does not change the physical state)
  arm_kernel<<<1, 1, 0, c->stream>>>(c->d_sc, 1e300);
  const DevView v = view(c);
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
  for (int e = 0; e < 5 && e < cap; ++e) ms[e] = c->phase_ms[e];
  if (n_phases) *n_phases = 5;
  return PSPH_OK;
}

int64_t psph_last_launch_count(const psph_ctx* c) { return c ? c->last_launches : 0; }

psph_status psph_step_timed(psph_ctx* c, int64_t nsteps, double* device_ms, int64_t* steps_done) {
  if (!c || !device_ms) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_step_timed before psph_upload");
  const bool was = c->timing;
  c->timing = false;
  cudaEvent_t e0, e1;
  CUDA_TRY(c, cudaEventCreate(&e0));
  CUDA_TRY(c, cudaEventCreate(&e1));
  // make sure the graph exists before the timed region
  if (!c->graph) {
    psph_status st = psph_step(c, 0, 1e300, nullptr);
    if (st) return st;
  }
  CUDA_TRY(c, cudaEventRecord(e0, c->stream));
  psph_status st = psph_step(c, nsteps, 1e300, steps_done);
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->timing = was;
  *device_ms = ms;
  return st;
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

}  // extern "C"

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
// device, by the first call on that device (with that device current); make
// that first call before any stream capture. Every call shares the array and
// overwrites what it needs (nothing in it has to start at zero); two calls
// whose work overlaps on the GPU (different streams, or contexts used from
// several threads) race on it.
// ---------------------------------------------------------------------------
namespace {

constexpr int kNoallocBlocks = (PSPH_NOALLOC_MAX_PARTICLES + 1023) / 1024 + 2;
// counts[MAX] | offsets[MAX + 1] | scan block sums
static __device__ __align__(256) int g_noalloc_scratch[2 * PSPH_NOALLOC_MAX_PARTICLES + 1 + kNoallocBlocks];

constexpr int kMaxDevices = 64;
int* g_noalloc_addr[kMaxDevices] = {};

psph_status noalloc_scratch(psph_ctx* c, int** out) {
  int dev = -1;
  CUDA_TRY(c, cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_err(c, PSPH_ERR_NO_DEVICE, "device index %d out of range", dev);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    CUDA_TRY(c, cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = (int*)p;
  }
  *out = g_noalloc_addr[dev];
  return PSPH_OK;
}

}  // namespace

extern "C" psph_status psph_pairs_export_noalloc(psph_ctx* c, int which, int64_t* pairs_device, int64_t cap,
                                                 int64_t* n_total) {
  if (!c || (which != 0 && which != 1) || cap < 0 || (cap > 0 && !pairs_device)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return set_err(c, PSPH_ERR_STATE, "psph_pairs_export_noalloc before psph_upload");
  if (c->ncap > PSPH_NOALLOC_MAX_PARTICLES)
    return set_err(c, PSPH_ERR_INVALID_ARGUMENT,
                   "psph_pairs_export_noalloc handles at most %d particles (context holds %d); use psph_pairs_export",
                   PSPH_NOALLOC_MAX_PARTICLES, c->ncap);
  int* scratch = nullptr;
  psph_status st = noalloc_scratch(c, &scratch);
  if (st) return st;
  int* counts = scratch;
  int* offsets = scratch + PSPH_NOALLOC_MAX_PARTICLES;
  int* block_sums = offsets + PSPH_NOALLOC_MAX_PARTICLES + 1;
  cudaStream_t s = c->stream;
  arm_kernel<<<1, 1, 0, s>>>(c->d_sc, 1e300);
  const DevView v = view(c);
  launch_sort(v, s);                                   // cell list of the current positions
  launch_pairs_count(v, which, counts, s);             // pairs each sorted particle lists first
  launch_exclusive_scan(counts, offsets, c->ncap, block_sums, s);
  launch_pairs_write(v, which, offsets, (long long*)pairs_device, (long long)cap, s);
  CUDA_TRY(c, cudaGetLastError());
  int total = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&total, offsets + c->ncap, sizeof(int), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(c, cudaStreamSynchronize(s));
  if (n_total) *n_total = total;
  return PSPH_OK;
}
