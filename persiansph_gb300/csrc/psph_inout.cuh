// In/out-flow boundaries: records exchanged between the host bookkeeping and
// the device kernels (psph_inout.cu).
#pragma once

#include "psph_device.cuh"

namespace psph {

// a candidate of the in-flow traversal: original index, cell, x
struct FlowCand {
  long long orig;
  int cx, cy, cz, pad;
  double x0;
};

// a particle's original index, current slot, class and position
struct FlowSlot {
  long long orig;
  int slot, cls;
  double x, y, z;
};

// one recycled in-flow particle: into a freed slot (append = 0) or appended at
// slot (append = 1) with original index orig and density (RefDensity of b);
// src_slot is the in-flow particle it copies
struct FlowRecycle {
  int slot, src_slot, cls, append;
  long long orig;
  double x, y, z, density;
};

// the state a user InCon / OutCon gave one particle (set_v / set_d: which
// parts to take)
struct FlowState {
  int slot, set_v, set_d, pad;
  double vx, vy, vz, den;
};

void flow_slot_of(const DevView& v, int n, int* slot_of, cudaStream_t st);
void flow_inflow_candidates(const DevView& v, int n, int qmax, double loc1, int need_io, int* count, FlowCand* out,
                            int cap, cudaStream_t st);
void flow_set_io(const DevView& v, const long long* origs, int m, const int* slot_of, int value, cudaStream_t st);
void flow_inflow_state(const DevView& v, const long long* origs, int m, const int* slot_of, const double* vel,
                       double den, cudaStream_t st);
void flow_outflow_mark(const DevView& v, int n, double out_loc, int* count, cudaStream_t st);
void flow_outflow_state(const DevView& v, int n, double out_loc, const double* vel, double den, int set_v, int set_d,
                        cudaStream_t st);
void flow_leaving(const DevView& v, int n, int* count, FlowSlot* out, int cap, cudaStream_t st);
void flow_gather_slots(const DevView& v, const long long* origs, int m, const int* slot_of, FlowSlot* out,
                       cudaStream_t st);
void flow_recycle(const DevView& v, const FlowRecycle* cmds, int m, cudaStream_t st);
void flow_outflow_list(const DevView& v, int n, double out_loc, int* count, FlowSlot* out, int cap,
                       cudaStream_t st);
void flow_apply(const DevView& v, const FlowState* states, int m, cudaStream_t st);

}  // namespace psph
