// Per-step neighbour lists (replaces the candidate arrays SMPairs / FSMPairs /
// NSMPairs of MainNeighbourSearch, Source/Domain.cpp:808-945).
//
// Each particle scans the sorted ranges of its 3x3(x3) cell block once per step
// (the rows and x-slabs of it that can reach the support) and keeps the
// candidates inside the kernel support, tested in FP32 on
// (cell offset, FP32 offset) separations with a margin on r^2 (0.02 % for the
// FP32C form, 0.4 % for the FP64 form); the pair kernels then apply the exact
// test of their form. Lists are written in 16-byte chunks of 4 entries, chunk-
// major across particles (nl_index), so a warp reading chunk c of 32
// consecutive particles touches 512 contiguous bytes and each store fills
// half a sector. The
// scan is cheap integer/FP32 work; the pair kernels then walk lists of nearly
// equal length instead of branching per candidate.
#include "psph_pairs.cuh"

namespace psph {

namespace {

constexpr int kNT = 128;

template <int DIM, bool UNIFORM_H>
__global__ void __launch_bounds__(kNT, 8) nlist_kernel(DevView v, float margin) {
  // Entries go through an 8-slot ring per lane, lane-interleaved (slot s of
  // lane l at ring[s][l], so the per-candidate stores are bank-conflict free);
  // the ring holds the chunk being filled and the next one, and a completed
  // chunk goes out as one 16-byte store.
  __shared__ int ring[8][kNT];
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
  // support test r^2 <= (Cellfac hb)^2 margin; with one h everywhere it is a constant
  const float thr_u = cf * cf * oi.w * oi.w * margin;
  const int N = v.ncap, cap = v.o.nl_cap;
  const CellCoord c = decode(g, cell);
  const float4* __restrict__ off = v.S.OFF32;
  int4* __restrict__ out = reinterpret_cast<int4*>(v.S.nl) + i;  // the next chunk to write; chunk c at nl + c * N + i
  int* const rp = &ring[0][threadIdx.x];                            // slot s at rp[s * kNT]
  // Rows of cells and x-slabs of cells whose nearest point lies outside the
  // support are skipped (cells are sorted slab by slab, xsub slabs along x).
  // The bound assumes the in-cell offset of i lies in [0, cell size), which
  // holds away from the grid faces (ListGenerate clamps only there); a
  // neighbour cell's clamped particles lie beyond its outer face, farther
  // from i than the slab they are counted in.
  const bool inner = c.x > 0 && c.x < g.nc[0] - 1 && c.y > 0 && c.y < g.nc[1] - 1 &&
                     (DIM == 2 || (c.z > 0 && c.z < g.nc[2] - 1));
  const bool cull = UNIFORM_H && inner;
  const float thr_cull = thr_u * 1.0001f;
  const int xs = v.o.xsub;
  const int* __restrict__ sstart = xs > 1 ? v.S.sstart : v.S.start;
  const float inv_sw = (float)xs / cs.x;  // 1 / slab width
  int k = 0;
  // the entry is written to the next free slot for every candidate and kept
  // (k advances) only when the candidate is inside
  auto put = [&](int e, bool in) {
    rp[(k & 7) * kNT] = e;
    k += in ? 1 : 0;
  };
  // after candidates that started at count k0 (at most 4 of them): the chunk
  // k0 / 4, if they completed it and it fits the capacity
  auto flush = [&](int k0) {
    if (((k0 ^ k) & 4) && k0 < cap) {
      const int b = (k0 & 4) * kNT;
      *out = make_int4(rp[b], rp[b + kNT], rp[b + 2 * kNT], rp[b + 3 * kNT]);
      out += N;
    }
  };
  const int zlo = (DIM == 3) ? -1 : 0, zhi = (DIM == 3) ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz) {
    int z = c.z + dz;
    if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
    else if (z < 0 || z >= g.nc[2]) continue;
    const float gz = (DIM == 3) ? (dz < 0 ? oi.z : (dz > 0 ? cs.z - oi.z : 0.f)) : 0.f;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = c.y + dy;
      if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
      else if (y < 0 || y >= g.nc[1]) continue;
      const float gy = dy < 0 ? oi.y : (dy > 0 ? cs.y - oi.y : 0.f);
      const int base = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
      const int cyz = 3 * (dy + 1) + 9 * (dz + 1);
      const float cy = -(float)dy * cs.y, cz = -(float)dz * cs.z;  // exact: dy, dz in {-1, 0, 1}
      // slabs in reach along x, counted from the first slab of i's cell
      int slo = -xs, shi = 2 * xs - 1;
      if (cull) {
        const float rx2 = thr_cull - gy * gy - gz * gz;
        if (rx2 < 0.f) continue;
        const float rx = sqrtf(rx2);
        slo = max(slo, (int)floorf((oi.x - rx) * inv_sw - 1e-3f));
        shi = min(shi, (int)floorf((oi.x + rx) * inv_sw + 1e-3f));
      }
      for (int dx = -1; dx <= 1; ++dx) {
        int x = c.x + dx;
        if (g.periodic[0]) x = (x + g.nc[0]) % g.nc[0];
        else if (x < 0 || x >= g.nc[0]) continue;
        const int s0 = max(slo - dx * xs, 0), s1 = min(shi - dx * xs, xs - 1);
        if (s0 > s1) continue;
        int lo = sstart[(base + x) * xs + s0];
        const int hi = sstart[(base + x) * xs + s1 + 1];
        const int tag = ((dx + 1) + cyz) << kCodeShift;
        // i's position relative to this cell's origin: x_i - x_j = a - off_j
        // (one rounding away from rel_pos's form, which the pair kernels
        // apply exactly; the list's margin covers the difference)
        const float ax = oi.x - (float)dx * cs.x, ay = oi.y + cy, az = oi.z + cz;
        auto inside = [&](int j) {
          const float4 oj = off[j];
          const float x0 = ax - oj.x, x1 = ay - oj.y, x2 = (DIM == 3) ? az - oj.z : 0.f;
          float thr = thr_u;
          if (!UNIFORM_H) {
            const float hb = 0.5f * (oi.w + oj.w);
            thr = cf * cf * hb * hb * margin;
          }
          return x0 * x0 + x1 * x1 + x2 * x2 <= thr;
        };
        auto one = [&](int j) {
          const int k0 = k;
          put(j | tag, inside(j));
          flush(k0);
        };
        if (dx == 0 && dy == 0 && dz == 0 && lo <= i && i < hi) {  // the home cell: skip i itself
          for (int j = lo; j < i; ++j) one(j);
          lo = i + 1;
        }
        int j = lo;
        for (; j + 4 <= hi; j += 4) {  // groups of 4: one chunk check per group
          const bool in0 = inside(j), in1 = inside(j + 1), in2 = inside(j + 2), in3 = inside(j + 3);
          const int k0 = k;
          put(j | tag, in0);
          put((j + 1) | tag, in1);
          put((j + 2) | tag, in2);
          put((j + 3) | tag, in3);
          flush(k0);
        }
        for (; j < hi; ++j) one(j);
      }
    }
  }
  if (k <= cap && (k & 3)) {  // last, partial chunk
    const int b = (k & 4) * kNT;
    *out = make_int4(rp[b], rp[b + kNT], rp[b + 2 * kNT], rp[b + 3 * kNT]);
  }
  v.S.nl_count[i] = (k <= cap) ? k : -1;
}

}  // namespace

void launch_nlist(const DevView& v, cudaStream_t st) {
  const int nb = v.ncap > 0 ? (v.ncap + kNT - 1) / kNT : 1;
  // a superset of the support: the pair kernels apply the exact test (FP32 in
  // the FP32C form, FP64 in the plain form)
  const float margin = v.o.fp32 ? 1.0002f : 1.004f;
  const bool uh = v.o.uniform_h;
  if (v.o.dim == 2) {
    if (uh) nlist_kernel<2, true><<<nb, kNT, 0, st>>>(v, margin);
    else nlist_kernel<2, false><<<nb, kNT, 0, st>>>(v, margin);
  } else {
    if (uh) nlist_kernel<3, true><<<nb, kNT, 0, st>>>(v, margin);
    else nlist_kernel<3, false><<<nb, kNT, 0, st>>>(v, margin);
  }
}

}  // namespace psph
