// Neighbour iteration shared by the pair kernels: cell decoding, the
// reference's periodic correction and pair orientation, the candidate stream
// over the 3x3(x3) block of cells, and FP32 relative positions from
// (cell offset, FP32 offset within the cell).
#pragma once

#include <cfloat>
#include <climits>

#include "psph_device.cuh"

namespace psph {

constexpr int kCodeShift = 26;  // neighbour-list entry: index | code << 26 (index < 2^26)
constexpr int kIndexMask = (1 << kCodeShift) - 1;

// Neighbour-list layout: chunks of 4 consecutive entries of one particle (16
// bytes), chunk-major across particles: chunk c of particle i is int4 number
// c * stride + nl_slot(i), so entry k sits at ((k / 4) * stride + nl_slot(i)) * 4
// + k % 4. Inside each block of 64 particles the even ones take slots 0-31 and
// the odd ones slots 32-63: the list scan, whose lanes own particles 2t and
// 2t+1, stores chunk c of a warp's even (odd) particles as 512 contiguous
// bytes, and a reader warp of 32 consecutive particles loads two runs of 256
// bytes; every access covers whole 32-byte sectors. stride = capacity rounded
// up to a multiple of 64.
PSPH_HD int nl_slot(int i) { return (i & ~63) | ((i & 1) << 5) | ((i >> 1) & 31); }
PSPH_HD size_t nl_index(int stride, int i, int k) {
  return (((size_t)(k >> 2) * stride + nl_slot(i)) << 2) + (k & 3);
}

struct CellCoord {
  int x, y, z;
};

// Cell coordinates of a global cell id within its instance's grid.
PSPH_D CellCoord decode(const GridDev& g, int c) {
  c -= g.cell_base;
  CellCoord r;
  r.x = c % g.nc[0];
  const int t = c / g.nc[0];
  r.y = t % g.nc[1];
  r.z = t / g.nc[1];
  return r;
}

// Periodic_X_Correction (Source/Domain.cpp:110-115) for the pair (P1, P2).
PSPH_D void periodic_fix(const GridDev& g, double& x0, double& x1, double& x2, double hb, const CellCoord& c1,
                         const CellCoord& c2) {
  const double lim = 2 * g.cellfac * hb;
  if (g.dom_size[0] > 0.0 && (x0 > lim || x0 < -lim)) x0 += (c1.x > c2.x) ? -g.dom_size[0] : g.dom_size[0];
  if (g.dom_size[1] > 0.0 && (x1 > lim || x1 < -lim)) x1 += (c1.y > c2.y) ? -g.dom_size[1] : g.dom_size[1];
  if (g.dom_size[2] > 0.0 && (x2 > lim || x2 < -lim)) x2 += (c1.z > c2.z) ? -g.dom_size[2] : g.dom_size[2];
}

// Visits the sorted index ranges of the 3 (2D) or 9 (3D) cell rows around c.
template <int DIM, class F>
PSPH_D void for_neighbor_ranges(const GridDev& g, const CellCoord& c, const int* __restrict__ start, F&& f) {
  const int zlo = (DIM == 3) ? -1 : 0, zhi = (DIM == 3) ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz) {
    int z = c.z + dz;
    if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
    else if (z < 0 || z >= g.nc[2]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = c.y + dy;
      if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
      else if (y < 0 || y >= g.nc[1]) continue;
      const int row = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
      if (!g.periodic[0] || (c.x >= 1 && c.x <= g.nc[0] - 2)) {
        const int x0 = max(c.x - 1, 0), x1 = min(c.x + 1, g.nc[0] - 1);
        f(start[row + x0], start[row + x1 + 1]);
      } else {
        for (int dx = -1; dx <= 1; ++dx) {
          const int x = (c.x + dx + g.nc[0]) % g.nc[0];
          f(start[row + x], start[row + x + 1]);
        }
      }
    }
  }
}

// True when MainNeighbourSearch lists (w, f) with w first: f's cell is in w's
// forward half stencil (Source/Domain.cpp:860-940), or, in the same cell, w
// has the larger index (head insertion reverses index order, :736-740).
PSPH_D bool first_of_pair(const GridDev& g, const CellCoord& cw, const CellCoord& cf, int orig_w, int orig_f) {
  int o[3] = {cf.x - cw.x, cf.y - cw.y, cf.z - cw.z};
  const int n[3] = {g.nc[0], g.nc[1], g.nc[2]};
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (g.periodic[d]) {
      if (o[d] > 1) o[d] -= n[d];
      if (o[d] < -1) o[d] += n[d];
    }
  if (o[2] != 0) return o[2] > 0;
  if (o[1] != 0) return o[1] > 0;
  if (o[0] != 0) return o[0] > 0;
  return orig_w > orig_f;
}

// The cell-offset code of two cells of the reference's grid packed as
// x | y << 10 | z << 20 (candidate minus home, each axis clamped to one cell:
// an in-support pair is never farther apart there).
PSPH_D int ref_code(int home, int cand) {
  const int dx = min(max((cand & 1023) - (home & 1023), -1), 1);
  const int dy = min(max(((cand >> 10) & 1023) - ((home >> 10) & 1023), -1), 1);
  const int dz = min(max((cand >> 20) - (home >> 20), -1), 1);
  return (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
}

// Same rule from a cell-offset code (candidate cell minus home cell, wrapped).
PSPH_D bool first_of_pair_code(int code, int orig_w, int orig_f) {
  const int dxc = code % 3 - 1, dyc = (code / 3) % 3 - 1, dzc = code / 9 - 1;
  if (dzc != 0) return dzc > 0;
  if (dyc != 0) return dyc > 0;
  if (dxc != 0) return dxc > 0;
  return orig_w > orig_f;
}

// Candidate stream over the 3x3(x3) cells around a home cell, one row split
// into its 3 cells where the periodic x axis wraps; reports each candidate's
// cell offset code (dx+1) + 3(dy+1) + 9(dz+1) relative to the home cell.
template <int DIM>
struct Cands32 {
  static constexpr int NR = (DIM == 3 ? 9 : 3) * 3;
  int cx, cy, cz, r, j, jend, base, code_yz, sub;
  bool wrapx;
  PSPH_D void init(const GridDev& g, int cell) {
    j = jend = 0;
    base = code_yz = sub = 0;
    cx = cy = cz = 0;
    wrapx = false;
    if (cell < 0) {
      r = NR;
      return;
    }
    const CellCoord c = decode(g, cell);
    cx = c.x;
    cy = c.y;
    cz = c.z;
    r = 0;
    wrapx = g.periodic[0] && (cx == 0 || cx == g.nc[0] - 1);
  }
  PSPH_D bool range(const GridDev& g, const int* __restrict__ start, int rr, int& lo, int& hi) {
    const int row = rr / 3;
    sub = rr - 3 * row;
    const int dz = (DIM == 3) ? row / 3 - 1 : 0;
    const int dy = row % 3 - 1;
    int z = cz + dz, y = cy + dy;
    if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
    else if (z < 0 || z >= g.nc[2]) return false;
    if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
    else if (y < 0 || y >= g.nc[1]) return false;
    base = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
    code_yz = 3 * (dy + 1) + 9 * (dz + 1);
    if (!wrapx) {
      if (sub) return false;
      const int x0 = max(cx - 1, 0), x1 = min(cx + 1, g.nc[0] - 1);
      lo = start[base + x0];
      hi = start[base + x1 + 1];
    } else {
      const int x = (cx + sub - 1 + g.nc[0]) % g.nc[0];
      lo = start[base + x];
      hi = start[base + x + 1];
    }
    return lo < hi;
  }
  PSPH_D int next(const GridDev& g, const int* __restrict__ start, const int* __restrict__ cellid, int* code) {
    while (j >= jend) {
      if (r >= NR) return -1;
      int lo, hi;
      if (range(g, start, r++, lo, hi)) {
        j = lo;
        jend = hi;
      }
    }
    const int jj = j++;
    const int dxj = wrapx ? (sub - 1) : (cellid[jj] - base - cx);
    *code = (dxj + 1) + code_yz;
    return jj;
  }
};

// x_i - x_j in FP32 from the cell-offset code (cell_j - cell_i) and the offsets.
template <int DIM>
PSPH_D void rel_pos(const float3& cs, const float4& oi, const float4& oj, int code, float& x0, float& x1, float& x2) {
  const int dxc = code % 3 - 1, dyc = (code / 3) % 3 - 1, dzc = code / 9 - 1;
  x0 = -(float)dxc * cs.x + (oi.x - oj.x);
  x1 = -(float)dyc * cs.y + (oi.y - oj.y);
  x2 = (DIM == 3) ? -(float)dzc * cs.z + (oi.z - oj.z) : 0.f;
}

PSPH_HD float3 cell_size_f(const GridDev& g) {
  return make_float3(g.cell_size32[0], g.cell_size32[1], g.cell_size32[2]);
}

}  // namespace psph

namespace psph {

// Neighbours of particle i for a pair kernel: its list entries, or, when the
// list overflowed its capacity (count -1), the same FP32 test run over the
// cell block directly. next() returns -1 when exhausted.
template <int DIM>
struct NbrSource {
  int i, cnt, k;
  Cands32<DIM> cs;
  float4 oi;
  float margin;
  const GridDev* g;
  PSPH_D void init(const DevView& v, const GridDev& grid, int i_, bool on, float margin_) {
    i = i_;
    k = 0;
    margin = margin_;
    g = &grid;
    cnt = on ? v.S.nl_count[i] : 0;
    if (on && cnt < 0) {
      cs.init(grid, v.S.cellid[i]);
      oi = v.S.OFF32[i];
    } else {
      cs.init(grid, -1);
    }
  }
  PSPH_D int next(const DevView& v, int* code) {
    if (cnt >= 0) {
      if (k >= cnt) return -1;
      const int e = v.S.nl[nl_index(v.nl_stride, i, k)];
      ++k;
      *code = e >> kCodeShift;
      return e & kIndexMask;
    }
    const float3 csz = cell_size_f(*g);
    const float cf = (float)g->cellfac;
    while (true) {
      const int j = cs.next(*g, v.S.start, v.S.cellid, code);
      if (j < 0) return -1;
      if (j == i) continue;
      const float4 oj = v.S.OFF32[j];
      float x0, x1, x2;
      rel_pos<DIM>(csz, oi, oj, *code, x0, x1, x2);
      const float hb = 0.5f * (oi.w + oj.w);
      if (x0 * x0 + x1 * x1 + x2 * x2 <= cf * cf * hb * hb * margin) return j;
    }
  }
};

}  // namespace psph

namespace psph {

// End of a pair kernel: folds each particle's acceleration time-step bound into
// its instance's running minimum (an atomic minimum on the ordered bits of a
// non-negative double, so the result does not depend on arrival order; NaN
// bounds never win, as the reference's comparison ignores them) and adds the
// block's pair count. One atomic per warp when the warp's particles share an
// instance, which is the case except at instance boundaries. BT is the block
// size, or 0 for a kernel whose block size is chosen at launch (cred then
// holds 32 entries).
template <int BT>
PSPH_D void block_dt_and_pairs(const DevView& v, int inst, bool active, double dtc, unsigned long long npair2,
                               double* red, unsigned long long* cred) {
  const unsigned full = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned act = __ballot_sync(full, active);
  if (act) {
    const int first = __shfl_sync(full, inst, __ffs(act) - 1);
    const bool uniform = __all_sync(full, !active || inst == first);
    if (uniform) {
      double m = active ? dtc : DBL_MAX;
      for (int off = 16; off > 0; off >>= 1) m = fmin(m, __shfl_down_sync(full, m, off));
      if (lane == 0 && m < DBL_MAX)
        atomicMin(&v.inst[first].dtmin_bits, (unsigned long long)__double_as_longlong(m));
    } else if (active && dtc < DBL_MAX) {
      atomicMin(&v.inst[inst].dtmin_bits, (unsigned long long)__double_as_longlong(dtc));
    }
  }
  for (int off = 16; off > 0; off >>= 1) npair2 += __shfl_down_sync(full, npair2, off);
  if (lane == 0) cred[tid >> 5] = npair2;
  __syncthreads();
  if (tid == 0) {
    unsigned long long c = 0;
    const int nw = BT > 0 ? BT / 32 : (int)(blockDim.x >> 5);  // BT = 0: the launch's block size
    for (int k = 0; k < nw; ++k) c += cred[k];
    if (c) atomicAdd(&v.sc->pairs_x2, c);
  }
  (void)red;
}


// FP32C form of the same: the candidates are FP32 values, so their minimum is
// taken in FP32 (FLT_MAX for none) and converted to double once per warp; a
// conversion is exact and monotonic, so the FP64 minimum is the same value.
PSPH_D void block_dt32_and_pairs(const DevView& v, int inst, bool active, float dtc, unsigned long long npair2,
                                 unsigned long long* cred) {
  const unsigned full = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned act = __ballot_sync(full, active);
  if (act) {
    const int first = __shfl_sync(full, inst, __ffs(act) - 1);
    const bool uniform = __all_sync(full, !active || inst == first);
    if (uniform) {
      float m = active ? dtc : FLT_MAX;
      for (int off = 16; off > 0; off >>= 1) m = fminf(m, __shfl_down_sync(full, m, off));
      if (lane == 0 && m < FLT_MAX)
        atomicMin(&v.inst[first].dtmin_bits, (unsigned long long)__double_as_longlong((double)m));
    } else if (active && dtc < FLT_MAX) {
      atomicMin(&v.inst[inst].dtmin_bits, (unsigned long long)__double_as_longlong((double)dtc));
    }
  }
  for (int off = 16; off > 0; off >>= 1) npair2 += __shfl_down_sync(full, npair2, off);
  if (lane == 0) cred[tid >> 5] = npair2;
  __syncthreads();
  if (tid == 0) {
    unsigned long long c = 0;
    const int nw = (int)(blockDim.x >> 5);
    for (int k = 0; k < nw; ++k) c += cred[k];
    if (c) atomicAdd(&v.sc->pairs_x2, c);
  }
}

}  // namespace psph
