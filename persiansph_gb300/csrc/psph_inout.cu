// In/out-flow boundaries (Source/Domain.cpp:1327-1635): the per-particle work
// on the device. The ordered lists of the reference (BC.InPart in its list
// order, DelPart in index order, AddPart in InPart order) are kept by the host
// code in psph_api.cu, which launches these kernels between the parts of a
// step: after the cell sort (InFlowBCFresh) and after the update
// (InFlowBCLeave). Particles are named by their original index ("orig"),
// which orders them as the reference's particle array does (appended
// particles take the next index, deletions keep the order of the rest).
#include "psph_device.cuh"
#include "psph_inout.cuh"
#include "psph_pairs.cuh"

namespace psph {
namespace {

constexpr int kIT = 256;

inline int blocks(int n) { return n > 0 ? (n + kIT - 1) / kIT : 1; }

__global__ void slot_of_kernel(DevView v, int* __restrict__ slot_of) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  slot_of[cur_persist(v).orig[s]] = s;
}

// Free particles of the cells with x index <= qmax whose x <= loc1 (and, when
// need_io, already in the in-flow state): the candidates of InFlowBCFresh's
// traversal, in any order (the host orders them).
__global__ void inflow_candidates_kernel(DevView v, int qmax, double loc1, int need_io, int* __restrict__ count,
                                         FlowCand* __restrict__ out, int cap) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  const Persist& P = cur_persist(v);
  const int cell = v.S.cellid[s];
  if (cell < 0 || !v.cls[P.cls[s]].is_free) return;
  const GridDev& g = grid_of(v, 0);
  const CellCoord cc = decode(g, cell);
  const double x0 = P.X4[s].x;
  if (cc.x > qmax || !(x0 <= loc1)) return;
  if (need_io && P.io[s] != 1) return;
  const int k = atomicAdd(count, 1);
  if (k < cap) {
    FlowCand f;
    f.orig = P.orig[s];
    f.cx = cc.x;
    f.cy = cc.y;
    f.cz = cc.z;
    f.x0 = x0;
    out[k] = f;
  }
}

__global__ void set_io_kernel(DevView v, const long long* __restrict__ origs, int m, const int* __restrict__ slot_of,
                              int value) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int s = slot_of[origs[k]];
  if (s >= 0) cur_persist(v).io[s] = value;
}

// The state InCon / OutCon give (the reference's default hooks InFlowCon and
// OutFlowCon, Source/Domain.cpp:35-45): v, va, vb; Density, Densitya,
// Densityb and the pressure of that density.
PSPH_D void set_flow_state(const DevView& v, int s, double vx, double vy, double vz, double den, bool set_v,
                           bool set_d) {
  const Persist& P = cur_persist(v);
  const PClass& C = v.cls[P.cls[s]];
  double4_32a X = P.X4[s], V = P.V4[s], H = P.H4[s];
  if (set_v) {
    V.x = vx; V.y = vy; V.z = vz;
    H.x = vx; H.y = vy; H.z = vz;  // vb (Modified Verlet) or va (leapfrog)
  }
  if (set_d) {
    X.w = den;
    H.w = den;
    V.w = eos(C.pres_eq, C.cs, C.p0, den, C.rho0);
  }
  P.X4[s] = X;
  P.V4[s] = V;
  P.H4[s] = H;
  if (P.H4b) {  // leapfrog vb, Densityb
    double4_32a B = P.H4b[s];
    if (set_v) { B.x = vx; B.y = vy; B.z = vz; }
    if (set_d) B.w = den;
    P.H4b[s] = B;
  }
}

__global__ void inflow_state_kernel(DevView v, const long long* __restrict__ origs, int m,
                                    const int* __restrict__ slot_of, double vx, double vy, double vz, double den) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const int s = slot_of[origs[k]];
  if (s >= 0) set_flow_state(v, s, vx, vy, vz, den, true, true);
}

// OutPart: free particles at or beyond out_loc take the out-flow state flag
__global__ void outflow_mark_kernel(DevView v, double out_loc, int* __restrict__ count) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  const Persist& P = cur_persist(v);
  if (v.S.cellid[s] < 0 || !v.cls[P.cls[s]].is_free || !(P.X4[s].x >= out_loc)) return;
  P.io[s] = 2;
  atomicAdd(count, 1);
}

__global__ void outflow_state_kernel(DevView v, double out_loc, double vx, double vy, double vz, double den,
                                     int set_v, int set_d) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  const Persist& P = cur_persist(v);
  if (v.S.cellid[s] < 0 || P.io[s] != 2 || !v.cls[P.cls[s]].is_free || !(P.X4[s].x >= out_loc)) return;
  set_flow_state(v, s, vx, vy, vz, den, set_v != 0, set_d != 0);
}

// the out-flow particles (those outflow_state_kernel sets), with their
// positions, for a user OutCon on the host
__global__ void outflow_list_kernel(DevView v, double out_loc, int* __restrict__ count, FlowSlot* __restrict__ out,
                                    int cap) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n) return;
  const Persist& P = cur_persist(v);
  if (v.S.cellid[s] < 0 || P.io[s] != 2 || !v.cls[P.cls[s]].is_free || !(P.X4[s].x >= out_loc)) return;
  const int k = atomicAdd(count, 1);
  if (k < cap) {
    FlowSlot f;
    f.orig = P.orig[s];
    f.slot = s;
    f.cls = P.cls[s];
    const double4_32a x = P.X4[s];
    f.x = x.x; f.y = x.y; f.z = x.z;
    out[k] = f;
  }
}

// the states a user InCon / OutCon returned, one per listed particle
__global__ void apply_states_kernel(DevView v, const FlowState* __restrict__ states, int m) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const FlowState f = states[k];
  if (f.slot >= 0 && f.slot < v.sc->n) set_flow_state(v, f.slot, f.vx, f.vy, f.vz, f.den, f.set_v != 0, f.set_d != 0);
}

// DelPart: the particles the update found outside the grid box, which leave
// the in/out-flow state
__global__ void leaving_kernel(DevView v, int* __restrict__ count, FlowSlot* __restrict__ out, int cap) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= v.sc->n || v.alive[s]) return;
  const Persist& P = cur_persist(v);
  P.io[s] = 0;
  const int k = atomicAdd(count, 1);
  if (k < cap) {
    FlowSlot f;
    f.orig = P.orig[s];
    f.slot = s;
    f.cls = P.cls[s];
    const double4_32a x = P.X4[s];
    f.x = x.x; f.y = x.y; f.z = x.z;
    out[k] = f;
  }
}

// slot, class and position of the listed particles
__global__ void gather_slots_kernel(DevView v, const long long* __restrict__ origs, int m,
                                    const int* __restrict__ slot_of, FlowSlot* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const Persist& P = cur_persist(v);
  const int s = slot_of[origs[k]];
  FlowSlot f;
  f.orig = origs[k];
  f.slot = s;
  f.cls = s >= 0 ? P.cls[s] : -1;
  const double4_32a x = s >= 0 ? P.X4[s] : make_double4_32a(0, 0, 0, 0);
  f.x = x.x; f.y = x.y; f.z = x.z;
  out[k] = f;
}

// Recycled in-flow particles: a freed slot takes the new position and class
// (its velocity and density stay until the next InCon, as in the reference);
// an appended particle is constructed as the reference's Particle(ID, x, v_b,
// Mass_b, RefDensity_b, h_b, false) with the fields copied from b.
__global__ void recycle_kernel(DevView v, const FlowRecycle* __restrict__ cmds, int m) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  const Persist& P = cur_persist(v);
  const FlowRecycle c = cmds[k];
  const int s = c.slot;
  if (c.append) {
    const double4_32a vb = P.V4[c.src_slot];
    P.X4[s] = make_double4_32a(c.x, c.y, c.z, c.density);
    P.V4[s] = make_double4_32a(vb.x, vb.y, vb.z, 0.0);
    P.H4[s] = make_double4_32a(0, 0, 0, 0);
    if (P.H4b) P.H4b[s] = make_double4_32a(0, 0, 0, 0);
    P.orig[s] = (int)c.orig;
  } else {
    double4_32a X = P.X4[s];
    X.x = c.x; X.y = c.y; X.z = c.z;
    P.X4[s] = X;
  }
  P.cls[s] = c.cls;
  P.io[s] = 1;
  if (P.mu) P.mu[s] = P.mu[c.src_slot];
  v.alive[s] = 1;
}

}  // namespace

void flow_slot_of(const DevView& v, int n, int* slot_of, cudaStream_t st) {
  slot_of_kernel<<<blocks(n), kIT, 0, st>>>(v, slot_of);
}
void flow_inflow_candidates(const DevView& v, int n, int qmax, double loc1, int need_io, int* count, FlowCand* out,
                            int cap, cudaStream_t st) {
  inflow_candidates_kernel<<<blocks(n), kIT, 0, st>>>(v, qmax, loc1, need_io, count, out, cap);
}
void flow_set_io(const DevView& v, const long long* origs, int m, const int* slot_of, int value, cudaStream_t st) {
  if (m > 0) set_io_kernel<<<blocks(m), kIT, 0, st>>>(v, origs, m, slot_of, value);
}
void flow_inflow_state(const DevView& v, const long long* origs, int m, const int* slot_of, const double* vel,
                       double den, cudaStream_t st) {
  if (m > 0) inflow_state_kernel<<<blocks(m), kIT, 0, st>>>(v, origs, m, slot_of, vel[0], vel[1], vel[2], den);
}
void flow_outflow_mark(const DevView& v, int n, double out_loc, int* count, cudaStream_t st) {
  outflow_mark_kernel<<<blocks(n), kIT, 0, st>>>(v, out_loc, count);
}
void flow_outflow_state(const DevView& v, int n, double out_loc, const double* vel, double den, int set_v, int set_d,
                        cudaStream_t st) {
  outflow_state_kernel<<<blocks(n), kIT, 0, st>>>(v, out_loc, vel[0], vel[1], vel[2], den, set_v, set_d);
}
void flow_leaving(const DevView& v, int n, int* count, FlowSlot* out, int cap, cudaStream_t st) {
  leaving_kernel<<<blocks(n), kIT, 0, st>>>(v, count, out, cap);
}
void flow_gather_slots(const DevView& v, const long long* origs, int m, const int* slot_of, FlowSlot* out,
                       cudaStream_t st) {
  if (m > 0) gather_slots_kernel<<<blocks(m), kIT, 0, st>>>(v, origs, m, slot_of, out);
}
void flow_recycle(const DevView& v, const FlowRecycle* cmds, int m, cudaStream_t st) {
  if (m > 0) recycle_kernel<<<blocks(m), kIT, 0, st>>>(v, cmds, m);
}
void flow_outflow_list(const DevView& v, int n, double out_loc, int* count, FlowSlot* out, int cap,
                       cudaStream_t st) {
  outflow_list_kernel<<<blocks(n), kIT, 0, st>>>(v, out_loc, count, out, cap);
}
void flow_apply(const DevView& v, const FlowState* states, int m, cudaStream_t st) {
  if (m > 0) apply_states_kernel<<<blocks(m), kIT, 0, st>>>(v, states, m);
}

}  // namespace psph
