// Per-step neighbour lists (replaces the candidate arrays SMPairs / FSMPairs /
// NSMPairs of MainNeighbourSearch, Source/Domain.cpp:808-945).
//
// Each particle scans the sorted ranges of its 3x3(x3) cell block once per step
// (the rows and x-slabs of it that can reach the support) and keeps the
// candidates inside the kernel support, tested in FP32 on
// (cell offset, FP32 offset) separations with a margin on r^2 (0.02 % for the
// FP32C form, 0.4 % for the FP64 form); the pair kernels then apply the exact
// test of their form. Lists are written in 16-byte chunks of 4 entries, chunk-
// major across particles (nl_index / nl_slot), so every store and every
// reader's load covers whole 32-byte sectors. The scan is cheap integer/FP32
// work; the pair kernels then walk lists of nearly equal length instead of
// branching per candidate.
//
// With one h everywhere (nlist_pair_kernel) a lane scans for two particles of
// one cell at once; otherwise (nlist_kernel) a lane scans for one particle.
//
// Staged form (nlist_staged_kernel, one h everywhere, x not periodic): a block
// first copies the candidate positions of its particles' neighbour cells into
// shared memory with TMA bulk copies, then scans them there. The block's 256
// particles are consecutive in cell order, so they occupy one row of cells
// (or the end of one row and the start of the next); for each such home row
// and each of the 3 (2D) or 9 (3D) neighbouring rows, the cells within one of
// the home cells' x-range form one contiguous range of sorted particles: one
// bulk copy each. A block whose ranges do not fit the staging buffer, or
// whose particles span more rows or instances, scans global memory as before.
#include <algorithm>

#include "psph_pairs.cuh"
#include "psph_tma.cuh"

namespace psph {

namespace {

constexpr int kNT = 128;

// Shared pieces of both scans. The 8-slot entry ring of a lane is
// lane-interleaved (slot s of lane l at ring[s][l], so the per-candidate
// stores are bank-conflict free); it holds the chunk being filled and the next
// one, and a completed chunk goes out as one 16-byte store.
struct ListWriter {
  int* rp;    // this lane's slot 0; slot s at rp[s * kNT]
  int4* out;  // the next chunk to write; chunk c of particle i at nl + c * stride + nl_slot(i)
  int k = 0;  // entries kept
  // the entry goes to the next free slot for every candidate and is kept (k
  // advances) only when the candidate is inside
  __device__ __forceinline__ void put(int e, bool in) {
    rp[(k & 7) * kNT] = e;
    k += in ? 1 : 0;
  }
  // after at most 4 candidates that started at count k0: the chunk k0 / 4, if
  // they completed it and it fits the capacity
  __device__ __forceinline__ void flush(int k0, int cap, int N) {
    if (((k0 ^ k) & 4) && k0 < cap) {
      const int b = (k0 & 4) * kNT;
      __stcs(out, make_int4(rp[b], rp[b + kNT], rp[b + 2 * kNT], rp[b + 3 * kNT]));
      out += N;
    }
  }
  __device__ __forceinline__ void finish(int cap, int* count) {
    if (k <= cap && (k & 3)) {  // last, partial chunk
      const int b = (k & 4) * kNT;
      __stcs(out, make_int4(rp[b], rp[b + kNT], rp[b + 2 * kNT], rp[b + 3 * kNT]));
    }
    *count = (k <= cap) ? k : -1;
  }
};

// Rows of cells and x-slabs of cells whose nearest point lies outside the
// support are skipped (cells are sorted slab by slab, xsub slabs along x).
// The bound assumes the in-cell offset lies in [0, cell size), which holds
// away from the grid faces (ListGenerate clamps only there); a neighbour
// cell's clamped particles lie beyond its outer face, farther than the slab
// they are counted in. Returns false when the row is out of reach, else the
// slabs in reach along x, counted from the first slab of the particle's cell.
__device__ __forceinline__ bool slab_reach(float ox, float gy, float gz, float thr_cull, float inv_sw, int* slo,
                                           int* shi) {
  const float rx2 = thr_cull - gy * gy - gz * gz;
  if (rx2 < 0.f) return false;
  const float rx = sqrtf(rx2);
  *slo = (int)floorf((ox - rx) * inv_sw - 1e-3f);
  *shi = (int)floorf((ox + rx) * inv_sw + 1e-3f);
  return true;
}

// One particle's list: the candidates of its 3x3(x3) cell block inside the
// support, tested in FP32 on (cell offset, FP32 offset) separations.
template <int DIM, bool UNIFORM_H>
__device__ __forceinline__ void list_one(const DevView& v, int i, float margin, int* rp) {
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
  const int N = v.nl_stride, cap = v.o.nl_cap;
  const CellCoord c = decode(g, cell);
  const float4* __restrict__ off = v.S.OFF32;
  ListWriter w{rp, reinterpret_cast<int4*>(v.S.nl) + nl_slot(i)};
  const bool inner = c.x > 0 && c.x < g.nc[0] - 1 && c.y > 0 && c.y < g.nc[1] - 1 &&
                     (DIM == 2 || (c.z > 0 && c.z < g.nc[2] - 1));
  const bool cull = UNIFORM_H && inner;
  const float thr_cull = thr_u * 1.0001f;
  const int xs = v.o.xsub;
  const int* __restrict__ sstart = xs > 1 ? v.S.sstart : v.S.start;
  const float inv_sw = (float)xs / cs.x;  // 1 / slab width
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
      int slo = -xs, shi = 2 * xs - 1;
      if (cull) {
        int lo_, hi_;
        if (!slab_reach(oi.x, gy, gz, thr_cull, inv_sw, &lo_, &hi_)) continue;
        slo = max(slo, lo_);
        shi = min(shi, hi_);
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
          const int k0 = w.k;
          w.put(j | tag, inside(j));
          w.flush(k0, cap, N);
        };
        if (dx == 0 && dy == 0 && dz == 0 && lo <= i && i < hi) {  // the home cell: skip i itself
          for (int j = lo; j < i; ++j) one(j);
          lo = i + 1;
        }
        int j = lo;
        for (; j + 4 <= hi; j += 4) {  // groups of 4: one chunk check per group
          const bool in0 = inside(j), in1 = inside(j + 1), in2 = inside(j + 2), in3 = inside(j + 3);
          const int k0 = w.k;
          w.put(j | tag, in0);
          w.put((j + 1) | tag, in1);
          w.put((j + 2) | tag, in2);
          w.put((j + 3) | tag, in3);
          w.flush(k0, cap, N);
        }
        for (; j < hi; ++j) one(j);
      }
    }
  }
  w.finish(cap, v.S.nl_count + i);
}

template <int DIM, bool UNIFORM_H>
__global__ void __launch_bounds__(kNT, 8) nlist_kernel(DevView v, float margin) {
  __shared__ int ring[8][kNT];
  if (v.sc->all_stop || !v.sc->rebuild) return;  // lists with a skin: kept from the last rebuild
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.sc->n) return;
  list_one<DIM, UNIFORM_H>(v, i, margin, &ring[0][threadIdx.x]);
}

// Where the scan reads a candidate's FP32 offset: global memory, or the
// block's staged copy (row k of the lane's home row: smem index j + delta[k]).
struct GlobalCands {
  const float4* __restrict__ off;
  __device__ __forceinline__ void home(int) {}
  __device__ __forceinline__ void row(int) {}
  __device__ __forceinline__ float4 at(int j) const { return off[j]; }
};
template <int RPH>
struct StagedCands {
  uint32_t sbase;     // shared address of the staged offsets
  const int* delta;   // smem index - global index, per home row (2) x neighbour row (RPH)
  int row_a;          // the first home row (z * ny + y); the second is the next one
  int hsel = 0, d = 0;
  __device__ __forceinline__ void home(int r) { hsel = (r == row_a) ? 0 : RPH; }
  __device__ __forceinline__ void row(int k) { d = delta[hsel + k]; }
  __device__ __forceinline__ float4 at(int j) const { return tma::lds128(sbase + 16u * (uint32_t)(j + d)); }
};

template <int DIM, class Cands>
__device__ __forceinline__ void scan_two(const DevView& v, int ia, int n, float margin, Cands cand,
                                         int (*ring)[8][kNT]);

// One h everywhere: a lane builds the lists of sorted particles 2t and 2t+1
// when they share a cell. Both scan the same cell block, so each candidate is
// loaded once and tested against both, and the rows and slabs walked are the
// union of the two particles' reach. The odd particles whose cell starts at
// them (listed by the sort, nl_rest of them in S.tmp_perm) get a lane of their
// own in the first nr blocks of the grid, which the hardware starts first, so
// their scans run beside the pairs instead of after them.
template <int DIM>
__global__ void __launch_bounds__(kNT, 8) nlist_pair_kernel(DevView v, float margin, int nr) {
  __shared__ int ring[2][8][kNT];
  const StepScalars* sc = v.sc;
  if (sc->all_stop || !sc->rebuild) return;
  if ((int)blockIdx.x < nr) {
    const int m = min(sc->nl_rest, v.ncap);
    for (int q = blockIdx.x * kNT + threadIdx.x; q < m; q += nr * kNT)
      list_one<DIM, true>(v, v.S.tmp_perm[q], margin, &ring[0][0][threadIdx.x]);
    return;
  }
  const int n = sc->n;
  const int t = (blockIdx.x - nr) * kNT + threadIdx.x;
  scan_two<DIM>(v, 2 * t, n, margin, GlobalCands{v.S.OFF32}, ring);
}

// The two-particle scan of sorted particles ia and ia + 1 (one lane).
template <int DIM, class Cands>
__device__ __forceinline__ void scan_two(const DevView& v, int ia, int n, float margin, Cands cand,
                                         int (*ring)[8][kNT]) {
  const int ib = ia + 1;
  if (ia >= n) return;
  const int cell = v.S.cellid[ia];
  const int cellb = ib < n ? v.S.cellid[ib] : -1;
  const bool pair = cell >= 0 && cellb == cell;
  if (ib < n && cellb < 0) v.S.nl_count[ib] = 0;  // in no cell (sorted after every cell)
  if (cell < 0) {
    v.S.nl_count[ia] = 0;
    return;
  }
  const Persist& P = cur_persist(v);
  const GridDev& g = grid_of(v, v.cls[P.cls[ia]].inst);
  const float3 cs = cell_size_f(g);
  // particle b far away when it is not paired: its tests always fail
  constexpr float kFar = 1e18f;
  const float4 oa = v.S.OFF32[ia];
  const float4 ob = pair ? v.S.OFF32[ib] : make_float4(kFar, kFar, kFar, oa.w);
  const float cf = (float)g.cellfac;
  const float thr = cf * cf * oa.w * oa.w * margin;
  const int N = v.nl_stride, cap = v.o.nl_cap;
  const CellCoord c = decode(g, cell);
  cand.home(c.z * g.nc[1] + c.y);
  int4* const nl4 = reinterpret_cast<int4*>(v.S.nl);
  ListWriter wa{&ring[0][0][threadIdx.x], nl4 + nl_slot(ia)};
  ListWriter wb{&ring[1][0][threadIdx.x], nl4 + nl_slot(ib)};
  const int zlo_ = (DIM == 3) ? -1 : 0;
  const bool cull = c.x > 0 && c.x < g.nc[0] - 1 && c.y > 0 && c.y < g.nc[1] - 1 &&
                    (DIM == 2 || (c.z > 0 && c.z < g.nc[2] - 1));
  const float thr_cull = thr * 1.0001f;
  const int xs = v.o.xsub;
  const int* __restrict__ sstart = xs > 1 ? v.S.sstart : v.S.start;
  const float inv_sw = (float)xs / cs.x;
  const int zlo = (DIM == 3) ? -1 : 0, zhi = (DIM == 3) ? 1 : 0;
  for (int dz = zlo; dz <= zhi; ++dz) {
    int z = c.z + dz;
    if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
    else if (z < 0 || z >= g.nc[2]) continue;
    const float gza = (DIM == 3) ? (dz < 0 ? oa.z : (dz > 0 ? cs.z - oa.z : 0.f)) : 0.f;
    const float gzb = (DIM == 3) ? (dz < 0 ? ob.z : (dz > 0 ? cs.z - ob.z : 0.f)) : 0.f;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = c.y + dy;
      if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
      else if (y < 0 || y >= g.nc[1]) continue;
      const float gya = dy < 0 ? oa.y : (dy > 0 ? cs.y - oa.y : 0.f);
      const float gyb = dy < 0 ? ob.y : (dy > 0 ? cs.y - ob.y : 0.f);
      const int base = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
      const int cyz = 3 * (dy + 1) + 9 * (dz + 1);
      const float cy = -(float)dy * cs.y, cz = -(float)dz * cs.z;
      cand.row(3 * (dz - zlo_) + (dy + 1));
      int slo = -xs, shi = 2 * xs - 1;
      if (cull) {  // the union of the two particles' reach
        int la, ha, lb, hb;
        const bool ra = slab_reach(oa.x, gya, gza, thr_cull, inv_sw, &la, &ha);
        const bool rb = pair && slab_reach(ob.x, gyb, gzb, thr_cull, inv_sw, &lb, &hb);
        if (!ra && !rb) continue;
        if (!ra) la = lb, ha = hb;
        else if (rb) la = min(la, lb), ha = max(ha, hb);
        slo = max(slo, la);
        shi = min(shi, ha);
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
        const float cx = -(float)dx * cs.x;
        const float axa = oa.x + cx, aya = oa.y + cy, aza = oa.z + cz;
        const float axb = ob.x + cx, ayb = ob.y + cy, azb = ob.z + cz;
        // both particles' separations in packed FP32x2 arithmetic: a - off_j
        // as fma(off_j, -1, a) (one rounding, the subtraction's), then the
        // squared distances, one instruction for both particles' values
        const float2 AX = make_float2(axa, axb), AY = make_float2(aya, ayb), AZ = make_float2(aza, azb);
        const float2 M1 = make_float2(-1.f, -1.f);
        auto test = [&](int j, bool& ina, bool& inb) {
          const float4 oj = cand.at(j);
          const float2 ex = __ffma2_rn(make_float2(oj.x, oj.x), M1, AX);
          const float2 ey = __ffma2_rn(make_float2(oj.y, oj.y), M1, AY);
          float2 d2 = __fmul2_rn(ex, ex);
          d2 = __ffma2_rn(ey, ey, d2);
          if (DIM == 3) {
            const float2 ez = __ffma2_rn(make_float2(oj.z, oj.z), M1, AZ);
            d2 = __ffma2_rn(ez, ez, d2);
          }
          ina = d2.x <= thr;
          inb = d2.y <= thr;
        };
        auto one = [&](int j, bool ena, bool enb) {
          bool ina, inb;
          test(j, ina, inb);
          const int ka = wa.k, kb = wb.k;
          wa.put(j | tag, ina && ena);
          wb.put(j | tag, inb && enb);
          wa.flush(ka, cap, N);
          wb.flush(kb, cap, N);
        };
        if (dx == 0 && dy == 0 && dz == 0) {  // the home cell: neither particle lists itself
          const int e0 = min(ia, hi);
          for (int j = lo; j < e0; ++j) one(j, true, true);
          if (lo <= ia && ia < hi) one(ia, false, true);
          int nx = ia + 1;
          if (pair) {
            if (lo <= ib && ib < hi) one(ib, true, false);
            nx = ib + 1;
          }
          lo = max(lo, nx);
        }
        int j = lo;
        for (; j + 4 <= hi; j += 4) {
          bool a0, a1, a2, a3, b0, b1, b2, b3;
          test(j, a0, b0);
          test(j + 1, a1, b1);
          test(j + 2, a2, b2);
          test(j + 3, a3, b3);
          const int ka = wa.k, kb = wb.k;
          wa.put(j | tag, a0);
          wa.put((j + 1) | tag, a1);
          wa.put((j + 2) | tag, a2);
          wa.put((j + 3) | tag, a3);
          wb.put(j | tag, b0);
          wb.put((j + 1) | tag, b1);
          wb.put((j + 2) | tag, b2);
          wb.put((j + 3) | tag, b3);
          wa.flush(ka, cap, N);
          wb.flush(kb, cap, N);
        }
        for (; j < hi; ++j) one(j, true, true);
      }
    }
  }
  wa.finish(cap, v.S.nl_count + ia);
  if (pair) wb.finish(cap, v.S.nl_count + ib);
}

// Staged form of nlist_pair_kernel (see the file header). Warp 0 plans the
// block's copies: the home rows of its particles and, per home row and
// neighbour row, the sorted range of the cells within one of the home cells'
// x-range; lane 0 arms the mbarrier with the total bytes and each planning lane
// issues its range's bulk copy. Every thread waits for the copies with a time
// limit; a thread whose wait gives up sets ST_STAGE_TIMEOUT, scans global
// memory instead, and waits again (bounded) before the block exits, so no copy
// lands in shared memory the block no longer owns.
constexpr unsigned long long kStageWaitNs = 1000000000ull;

template <int DIM>
__global__ void __launch_bounds__(kNT, 4) nlist_staged_kernel(DevView v, float margin, int nr, int cap_stage) {
  constexpr int RPH = (DIM == 3) ? 9 : 3;  // neighbour rows per home row
  __shared__ int ring[2][8][kNT];
  __shared__ int s_delta[2 * RPH];
  __shared__ int s_row_a, s_mode;
  __shared__ __align__(8) uint64_t s_bar;
  extern __shared__ float4 s_off[];
  StepScalars* sc = v.sc;
  if (sc->all_stop || !sc->rebuild) return;
  if ((int)blockIdx.x < nr) {
    const int m = min(sc->nl_rest, v.ncap);
    for (int q = blockIdx.x * kNT + threadIdx.x; q < m; q += nr * kNT)
      list_one<DIM, true>(v, v.S.tmp_perm[q], margin, &ring[0][0][threadIdx.x]);
    return;
  }
  const int n = sc->n;
  const int b = blockIdx.x - nr;
  const int p0 = 2 * b * kNT;
  if (threadIdx.x == 0) {
    tma::mbar_init(&s_bar, 1);
    tma::mbar_init_fence();
  }
  // plan (warp 0): lane q < nh * RPH owns the range of home row q / RPH and
  // neighbour row q % RPH
  int seg_lo = 0, cnt = 0, off = 0, total = 0;
  if (threadIdx.x < 32) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    const int last = min(p0 + 2 * kNT, min(n, sc->n_cells)) - 1;
    bool ok = p0 <= last;
    const int ca = ok ? v.S.cellid[p0] : -1, cl = ok ? v.S.cellid[last] : -1;
    ok = ok && ca >= 0 && cl >= 0;
    const Persist& P = cur_persist(v);
    const int inst = ok ? v.cls[P.cls[p0]].inst : 0;
    ok = ok && v.cls[P.cls[last]].inst == inst;
    const GridDev& g = grid_of(v, inst);
    ok = ok && !g.periodic[0];
    const CellCoord A = decode(g, ok ? ca : g.cell_base), L = decode(g, ok ? cl : g.cell_base);
    const int ra = A.z * g.nc[1] + A.y, rl = L.z * g.nc[1] + L.y;
    const int nh = (rl == ra) ? 1 : (rl == ra + 1 ? 2 : 0);
    ok = ok && nh > 0;
    if (ok && lane < nh * RPH) {
      const int h = lane / RPH, k = lane % RPH;
      const int hy = h ? L.y : A.y, hz = h ? L.z : A.z;
      const int xlo = h ? 0 : A.x, xhi = (nh == 1 || h) ? L.x : g.nc[0] - 1;
      const int dz = (DIM == 3) ? k / 3 - 1 : 0, dy = k % 3 - 1;
      int y = hy + dy, z = hz + dz;
      bool in = true;
      if (g.periodic[1]) y = (y + g.nc[1]) % g.nc[1];
      else if (y < 0 || y >= g.nc[1]) in = false;
      if (g.periodic[2]) z = (z + g.nc[2]) % g.nc[2];
      else if (z < 0 || z >= g.nc[2]) in = false;
      if (in) {
        const int base = g.cell_base + (z * g.nc[1] + y) * g.nc[0];
        seg_lo = v.S.start[base + max(xlo - 1, 0)];
        cnt = v.S.start[base + min(xhi + 1, g.nc[0] - 1) + 1] - seg_lo;
      }
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(full, incl, o);
      if (lane >= o) incl += y;
    }
    total = __shfl_sync(full, incl, 31);
    off = incl - cnt;
    ok = ok && total > 0 && total <= cap_stage;
    if (lane < 2 * RPH) s_delta[lane] = off - seg_lo;
    if (lane == 0) {
      s_row_a = ra;
      s_mode = ok;
    }
    if (!ok) cnt = 0;
  }
  __syncthreads();  // the plan and the initialised mbarrier
  const bool staged = s_mode;
  const uint32_t sbase = tma::smem_u32(s_off);
  if (staged && threadIdx.x < 32) {
    if (threadIdx.x == 0) tma::mbar_expect_tx(&s_bar, 16u * (uint32_t)total);
    __syncwarp();
    if (cnt > 0) tma::bulk_g2s(sbase + 16u * (uint32_t)off, v.S.OFF32 + seg_lo, 16u * (uint32_t)cnt, &s_bar);
  }
  bool use_stage = staged;
  if (staged && !tma::mbar_wait_bounded(&s_bar, 0, kStageWaitNs)) {
    atomicOr(&sc->status, ST_STAGE_TIMEOUT);
    use_stage = false;
  }
  const int t = b * kNT + threadIdx.x;
  if (use_stage) scan_two<DIM>(v, 2 * t, n, margin, StagedCands<RPH>{sbase, s_delta, s_row_a}, ring);
  else scan_two<DIM>(v, 2 * t, n, margin, GlobalCands{v.S.OFF32}, ring);
  if (staged && !use_stage) tma::mbar_wait_bounded(&s_bar, 0, kStageWaitNs);
}

// Deepest staging (Options::nlist_stage): 64 KB of FP32 offsets per block
// (one home row of ~256 particles and its neighbour rows take ~2,600 in the
// 3D dam break).
constexpr int kStageCapMax = 4096;

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

}  // namespace

void nlist_configure() {
  const int bytes = kStageCapMax * (int)sizeof(float4);
  cudaFuncSetAttribute(nlist_staged_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  cudaFuncSetAttribute(nlist_staged_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

void launch_nlist(const DevView& v, cudaStream_t st) {
  // a superset of the support: the pair kernels apply the exact test (FP32 in
  // the FP32C form, FP64 in the plain form)
  // with a skin s the lists hold every pair within (1 + s) of the support
  const float margin = v.o.fp32 ? 1.0002f * (1.f + v.o.skin) * (1.f + v.o.skin) : 1.004f;
  if (v.o.uniform_h) {  // two particles per lane; the leftovers' blocks first
    const int half = (v.ncap + 1) / 2;
    const int nr = 2 * sm_count();
    const int nb = nr + (half > 0 ? (half + kNT - 1) / kNT : 1);
    const int cap = min(v.o.nlist_stage, kStageCapMax);
    if (cap > 0 && !v.o.any_periodic_x) {
      const size_t smem = (size_t)cap * sizeof(float4);
      if (v.o.dim == 2) nlist_staged_kernel<2><<<nb, kNT, smem, st>>>(v, margin, nr, cap);
      else nlist_staged_kernel<3><<<nb, kNT, smem, st>>>(v, margin, nr, cap);
      return;
    }
    if (v.o.dim == 2) nlist_pair_kernel<2><<<nb, kNT, 0, st>>>(v, margin, nr);
    else nlist_pair_kernel<3><<<nb, kNT, 0, st>>>(v, margin, nr);
    return;
  }
  const int nb = v.ncap > 0 ? (v.ncap + kNT - 1) / kNT : 1;
  if (v.o.dim == 2) nlist_kernel<2, false><<<nb, kNT, 0, st>>>(v, margin);
  else nlist_kernel<3, false><<<nb, kNT, 0, st>>>(v, margin);
}

}  // namespace psph
