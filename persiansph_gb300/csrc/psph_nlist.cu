// Per-step neighbour lists (replaces the candidate arrays SMPairs / FSMPairs /
// NSMPairs of MainNeighbourSearch, Source/Domain.cpp:808-945).
//
// Each particle scans the sorted ranges of its 3x3(x3) cell block once per step
// and keeps the candidates inside the kernel support, tested in FP32 on
// (cell offset, FP32 offset) separations: exactly for the FP32C form, with a
// 0.4 % margin on r^2 for the FP64 form (whose pair kernel then applies the
// exact FP64 test). Lists are laid out entry-major (nl[k*ncap + i]) so a warp
// reading entry k of 32 consecutive particles touches consecutive words. The
// scan is cheap integer/FP32 work; the pair kernels then walk lists of nearly
// equal length instead of branching per candidate.
#include "psph_pairs.cuh"

namespace psph {

namespace {

constexpr int kNT = 128;

template <int DIM>
__global__ void __launch_bounds__(kNT) nlist_kernel(DevView v, float margin) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc->n) return;
  const int cell = v.S.cellid[i];
  if (cell < 0) {
    v.S.nl_count[i] = 0;
    return;
  }
  const Persist& P = cur_persist(v);
  const GridDev& g = grid_of(v, v.cls[P.cls[i]].inst);
  const float3 cs = cell_size_f(g);
  const float4 oi = v.S.OFF32[i];
  const float cf = (float)g.cellfac;
  const int N = v.ncap, cap = v.o.nl_cap;
  const CellCoord c = decode(g, cell);
  const bool wrapx = g.periodic[0] && (c.x == 0 || c.x == g.nc[0] - 1);
  int* __restrict__ out = v.S.nl + i;
  int k = 0;
  const int zlo = (DIM == 3) ? -1 : 0, zhi = (DIM == 3) ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz) {
    int z = c.z + dz;
    if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
    else if (z < 0 || z >= g.nc[2]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = c.y + dy;
      if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
      else if (y < 0 || y >= g.nc[1]) continue;
      const int base = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
      const int cyz = 3 * (dy + 1) + 9 * (dz + 1);
      for (int sub = 0; sub < (wrapx ? 3 : 1); ++sub) {
        int lo, hi;
        if (!wrapx) {
          lo = v.S.start[base + max(c.x - 1, 0)];
          hi = v.S.start[base + min(c.x + 1, g.nc[0] - 1) + 1];
        } else {
          const int x = (c.x + sub - 1 + g.nc[0]) % g.nc[0];
          lo = v.S.start[base + x];
          hi = v.S.start[base + x + 1];
        }
        for (int j = lo; j < hi; ++j) {
          const int dxc = wrapx ? sub - 1 : v.S.cellid[j] - base - c.x;
          const int code = (dxc + 1) + cyz;
          const float4 oj = v.S.OFF32[j];
          float x0, x1, x2;
          rel_pos<DIM>(cs, oi, oj, code, x0, x1, x2);
          const float hb = 0.5f * (oi.w + oj.w);
          if (x0 * x0 + x1 * x1 + x2 * x2 <= cf * cf * hb * hb * margin && j != i) {
            if (k < cap) out[(size_t)k * N] = j | (code << kCodeShift);
            ++k;
          }
        }
      }
    }
  }
  v.S.nl_count[i] = (k <= cap) ? k : -1;
}

}  // namespace

void launch_nlist(const DevView& v, cudaStream_t st) {
  const int nb = v.ncap > 0 ? (v.ncap + kNT - 1) / kNT : 1;
  const float margin = v.o.fp32 ? 1.0f : 1.004f;
  if (v.o.dim == 2) nlist_kernel<2><<<nb, kNT, 0, st>>>(v, margin);
  else nlist_kernel<3><<<nb, kNT, 0, st>>>(v, margin);
}

}  // namespace psph
