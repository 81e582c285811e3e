// Cell list as a deterministic counting sort (replaces CellReset + ListGenerate,
// Source/Domain.cpp:662-806, and the per-step pair arrays of MainNeighbourSearch).
//
//   bin      cell key per particle, exactly ListGenerate's floor/clamp rule;
//            each cell is split into xsub slabs along x (the key counts
//            slabs: cell * xsub + slab), so the particles of a cell lie in
//            x-slab order and the neighbour-list walk can skip slabs out of
//            reach; key = nbins (= ncells * xsub) for a particle that
//            ListGenerate would drop into a periodic ghost column (it then
//            sits in no list), nbins+1 for one that CheckParticleLeave removed.
//   scan     exclusive prefix of the per-cell counts (3-phase, block-level).
//   scatter  atomic slot inside its cell's segment.
//   rank     deterministic order inside each slab: by original index, so the
//            sorted state depends only on positions, never on atomic timing.
//   starts   per-cell segment starts (start[c] = slab start of c's first slab)
//            for everything that walks whole cells, and the particles the
//            neighbour-list scan handles one per lane.
//   reorder  gathers every persistent field into the new order (HBM-bound).
#include <cstdio>

#include "psph_device.cuh"

namespace psph {

namespace {

constexpr int kBT = 256;

__global__ void bin_kernel(DevView v, const uint8_t* __restrict__ alive, int* __restrict__ key,
                           int* __restrict__ count, StepScalars* sc, int dim, int xsub) {
  if (sc->all_stop || !sc->rebuild) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int nbins = v.total_cells * xsub;
  const int orphan_key = nbins, dead_key = nbins + 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int k;
    if (!alive[i]) {
      k = dead_key;
    } else {
      const GridDev& g = grid_of(v, v.cls[P.cls[i]].inst);
      const double4_32a x = P.X4[i];
      const double xs[3] = {x.x, x.y, x.z};
      int c[3] = {0, 0, 0};
      double a0 = 0.0;  // x - BLPF_x
      bool orphan = false, out = false;
      for (int d = 0; d < dim; ++d) {
        // ListGenerate's floor((x - BLPF) / CellSize) (Source/Domain.cpp:669-691).
        // An FP32 estimate (the difference converted on the integer pipe)
        // decides it unless the quotient lies within the estimate's error of
        // an integer; only then the FP64 division runs (a division costs tens
        // of operations on the FP64 pipe).
        const double a = xs[d] - g.blpf[d];
        if (d == 0) a0 = a;
        const float t = d2f_bits(a) * g.inv_cell_size32[d];
        const float ft = floorf(t), fr = t - ft, tol = 1e-3f + 4e-7f * fabsf(t);
        int cd = (int)ft;
        if (!(fr >= tol && fr <= 1.f - tol)) cd = (int)floor(a / g.cell_size[d]);
        if (cd < 0) {
          if ((g.blpf[d] - xs[d]) <= g.hmax) cd = 0;
          else out = true;
        }
        if (cd >= g.cn_ref[d]) {
          if ((xs[d] - g.trpr[d]) <= g.hmax) cd = g.cn_ref[d] - 1;
          else out = true;
        }
        if (cd >= g.nc[d]) orphan = true;  // periodic ghost column: overwritten by the copy
        c[d] = cd;
      }
      if (out) {
        atomicOr(&sc->status, ST_OUT_OF_GRID);
        k = dead_key;
      } else if (orphan) {
        k = orphan_key;
      } else {
        int slab = 0;
        if (xsub > 1) {  // x-slab inside the cell (clamped for particles outside it), in FP32
          const float ox = d2f_bits(a0) - (float)c[0] * g.cell_size32[0];
          slab = min(max((int)floorf(ox * (float)xsub * g.inv_cell_size32[0]), 0), xsub - 1);
        }
        k = (g.cell_base + (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0]) * xsub + slab;
      }
    }
    key[i] = k;
    // one atomic per distinct cell of the warp: consecutive particles (sorted
    // by the previous step) mostly share their cell
    const unsigned peers = __match_any_sync(__activemask(), k);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&count[k], __popc(peers));
  }
}

// Phase 1: in-block exclusive scan of `in` (len entries), block totals to sums.
__global__ void scan_blocks(const int* __restrict__ in, int* __restrict__ out, int* __restrict__ sums, int len,
                            const StepScalars* sc) {
  if (sc && (sc->all_stop || !sc->rebuild)) return;  // the cell sort's scan, on a step without a rebuild
  __shared__ int warp_tot[32];
  const int base = blockIdx.x * 1024;
  const int t = threadIdx.x;
  const int i = base + t;
  int v = (i < len) ? in[i] : 0;
  const int lane = t & 31, w = t >> 5;
  int incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int s = warp_tot[lane];
    int si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += y;
    }
    warp_tot[lane] = si - s;  // exclusive warp offsets
    if (lane == 31) sums[blockIdx.x] = si;
  }
  __syncthreads();
  if (i < len) out[i] = incl - v + warp_tot[w];
}

// Phase 2: one block scans the block totals (exclusive), writes the grand total.
__global__ void scan_sums(int* __restrict__ sums, int nb, int* __restrict__ total_out, const StepScalars* sc) {
  if (sc && (sc->all_stop || !sc->rebuild)) return;
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int t = threadIdx.x, i = base + t;
    int v = (i < nb) ? sums[i] : 0;
    const int lane = t & 31, w = t >> 5;
    __shared__ int wt[32];
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wt[w] = incl;
    __syncthreads();
    if (w == 0) {
      int s = wt[lane], si = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, si, o);
        if (lane >= o) si += y;
      }
      wt[lane] = si - s;
    }
    __syncthreads();
    int excl = incl - v + wt[w] + carry;
    if (i < nb) sums[i] = excl;
    __syncthreads();
    if (t == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void scan_add(int* __restrict__ out, const int* __restrict__ sums, int len, const StepScalars* sc) {
  if (sc && (sc->all_stop || !sc->rebuild)) return;
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < len) out[i] += sums[blockIdx.x];
}

__global__ void scatter_kernel(const int* __restrict__ key, const int* __restrict__ start, int* __restrict__ fill,
                               int* __restrict__ tmp_perm, const StepScalars* sc) {
  if (sc->all_stop || !sc->rebuild) return;
  const int n = sc->n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = key[i];
    // warp-aggregated slot claim (the order inside a cell is fixed by rank_kernel)
    const unsigned peers = __match_any_sync(__activemask(), k);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&fill[k], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    tmp_perm[start[k] + base + __popc(peers & ((1u << lane) - 1u))] = i;
  }
}

__global__ void rank_kernel(const int* __restrict__ key, const int* __restrict__ start,
                            const int* __restrict__ tmp_perm, DevView v, int* __restrict__ perm,
                            const StepScalars* sc, int ncells) {
  if (sc->all_stop || !sc->rebuild) return;
  const int* __restrict__ orig = cur_persist(v).orig;
  const int n = sc->n;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const int i = tmp_perm[s];
    const int k = key[i];
    if (k <= ncells) {
      const int lo = start[k], hi = start[k + 1];
      const int mine = orig[i];
      int r = 0;
      for (int t = lo; t < hi; ++t) r += (orig[tmp_perm[t]] < mine);
      perm[lo + r] = i;
    } else {
      perm[s] = i;
    }
  }
}

__global__ void reorder_kernel(DevView v, const int* __restrict__ perm, const int* __restrict__ key,
                               const int* __restrict__ start, int* __restrict__ cellid, uint8_t* __restrict__ alive,
                               const StepScalars* sc, int nbins, int xsub, int has_solid, int dyn_mu) {
  if (sc->all_stop || !sc->rebuild) return;
  const Persist& src = cur_persist(v);
  const Persist& dst = next_persist(v);
  const int n_new = start[nbins + 1];
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n_new; s += gridDim.x * blockDim.x) {
    const int i = perm[s];
    dst.X4[s] = src.X4[i];
    dst.V4[s] = src.V4[i];
    dst.H4[s] = src.H4[i];
    if (src.H4b) dst.H4b[s] = src.H4b[i];
    dst.cls[s] = src.cls[i];
    {
      // FP32 offset from the cell origin (absolute position outside any cell)
      const double4_32a xs = src.X4[i];
      const int kk = key[i];
      const float h = (float)v.cls[src.cls[i]].h;
      if (kk < nbins) {
        const GridDev& g = grid_of(v, v.cls[src.cls[i]].inst);
        const int lk = kk / xsub - g.cell_base;
        const int cx = lk % g.nc[0], t = lk / g.nc[0], cy = t % g.nc[1], cz = t / g.nc[1];
        v.S.OFF32[s] = make_float4((float)(xs.x - (g.blpf[0] + cx * g.cell_size[0])),
                                   (float)(xs.y - (g.blpf[1] + cy * g.cell_size[1])),
                                   (float)(v.o.dim == 3 ? xs.z - (g.blpf[2] + cz * g.cell_size[2]) : 0.0), h);
      } else {
        v.S.OFF32[s] = make_float4((float)xs.x, (float)xs.y, (float)xs.z, h);
      }
      if (v.o.skin > 0.f)  // displacements are measured from here (FP32, truncated)
        v.S.OFFREF[s] = make_float4(d2f_bits(xs.x), d2f_bits(xs.y), d2f_bits(xs.z), 0.f);
    }
    dst.orig[s] = src.orig[i];
    if (src.io) dst.io[s] = src.io[i];
    const int k = key[i];
    cellid[s] = (k < nbins) ? k / xsub : -1;
    alive[s] = 1;
    if (dyn_mu) dst.mu[s] = src.mu[i];
  }
}

// The 3x3 tensors of solids (9 doubles a row) in the new order, a warp per 32
// rows: lane l moves words l, l+32, ... of the warp's 288, so the stores are
// contiguous and the loads too wherever the permutation keeps neighbours
// together (it mostly does: particles move little between steps).
__global__ void reorder_tensors_kernel(DevView v, const int* __restrict__ perm, const int* __restrict__ start,
                                       const StepScalars* sc, int nbins) {
  if (sc->all_stop || !sc->rebuild) return;
  const Persist& src = cur_persist(v);
  const Persist& dst = next_persist(v);
  const int n_new = start[nbins + 1];
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const double* srcs[7] = {src.sigma, src.sigma_h, src.strain, src.strain_h, src.shear, src.tir, src.shear_h};
  double* dsts[7] = {dst.sigma, dst.sigma_h, dst.strain, dst.strain_h, dst.shear, dst.tir, dst.shear_h};
  // the ShearStress history serves Mat2 only (a zero history of a soil domain stays behind)
  const int nt = v.o.carry_shear_h ? 7 : 6;
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; 32 * w < n_new; w += nwarps) {
    const int base = 32 * w;
    const int rows = min(32, n_new - base);
    const int mine = lane < rows ? perm[base + lane] : 0;  // the source row of this lane's destination row
    for (int a = 0; a < nt; ++a) {
      const double* __restrict__ sa = srcs[a];
      double* __restrict__ da = dsts[a] + 9 * (size_t)base;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const int word = lane + 32 * k;       // of the warp's 288
        const int r = word / 9, e = word - 9 * r;
        const int from = __shfl_sync(0xffffffffu, mine, r & 31);
        if (r < rows) da[word] = sa[9 * (size_t)from + e];
      }
    }
  }
}

__global__ void finish_sort_kernel(const int* __restrict__ start, StepScalars* sc, int nbins) {
  if (sc->all_stop || !sc->rebuild) return;
  sc->n_cells = start[nbins];
  sc->n = start[nbins + 1];
  sc->buf ^= 1;
  sc->nl_rest = 0;
}

// Per-cell segment starts from the slab starts (split cells): start[c] =
// sstart[c * xsub] for c <= ncells, and the orphan / dead / total boundaries
// after them. Also lists the particles the two-per-lane neighbour-list scan
// leaves to a lane of their own: lanes take sorted particles 2t and 2t+1
// together when they share a cell, so the odd particles left are exactly the
// cells' first particles at odd indices (into rest, at most cap of them).
__global__ void cell_starts_kernel(const int* __restrict__ sstart, int* __restrict__ start, int ncells, int xsub,
                                   StepScalars* sc, int* __restrict__ rest, int cap) {
  if (sc->all_stop || !sc->rebuild) return;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (xsub > 1) {
    if (c <= ncells) start[c] = sstart[(size_t)c * xsub];
    else if (c <= ncells + 2) start[c] = sstart[(size_t)ncells * xsub + (c - ncells)];
  }
  bool odd_first = false;
  int s0 = 0;
  if (c < ncells) {
    s0 = sstart[(size_t)c * xsub];
    odd_first = (s0 & 1) && sstart[(size_t)(c + 1) * xsub] > s0;
  }
  const unsigned want = __ballot_sync(0xffffffffu, odd_first);  // every lane of the grid gets here
  if (odd_first) {  // one atomic per warp
    const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&sc->nl_rest, __popc(want));
    base = __shfl_sync(want, base, leader);
    const int slot = base + __popc(want & ((1u << lane) - 1u));
    if (slot < cap) rest[slot] = s0;
  }
}

// Neighbour lists with a skin: on every step the FP32 offsets of the
// particles from their cells' origins (the cells of the last rebuild), and
// each particle's cell in the reference's grid (ListGenerate's floor and
// clamp on the FP64 position, Source/Domain.cpp:669-691), which orients the
// wall pressure's pairs as the reference's neighbour search does.
__global__ void skin_offsets_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sc->n) return;
  const Persist& P = cur_persist(v);
  const PClass& C = v.cls[P.cls[s]];
  const double4_32a xs = P.X4[s];
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
  const GridDev& r = v.grids_ref[C.inst];
  const double xd[3] = {xs.x, xs.y, xs.z};
  int q[3] = {0, 0, 0};
  for (int d = 0; d < v.o.dim; ++d) {
    // floor((x - BLPF) / CellSize) from an FP32 estimate, with the FP64
    // division only near a cell face (as the sort's bin_kernel)
    const double a = xd[d] - r.blpf[d];
    const float t = d2f_bits(a) * r.inv_cell_size32[d];
    const float ft = floorf(t), fr = t - ft, tol = 1e-3f + 4e-7f * fabsf(t);
    int k = (int)ft;
    if (!(fr >= tol && fr <= 1.f - tol)) k = (int)floor(a / r.cell_size[d]);
    q[d] = min(max(k, 0), r.cn_ref[d] - 1);  // clamped as ListGenerate clamps the particles just outside
  }
  v.S.refcell[s] = q[0] | (q[1] << 10) | (q[2] << 20);
}

// now: the next cell sort runs (a sort outside the step loop); next_step:
// the next step sorts and lists again (with a skin, whose lists would
// otherwise be kept)
__global__ void mark_rebuild_kernel(StepScalars* sc, int now, int next_step) {
  if (now) sc->rebuild = 1;
  if (next_step) sc->force_rebuild = 1;
}

inline int grid_for(int n) {
  int b = (n + kBT - 1) / kBT;
  return b < 1 ? 1 : b;
}

}  // namespace

void launch_skin_offsets(const DevView& v, cudaStream_t st) {
  skin_offsets_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(v);
}

void launch_mark_rebuild(const DevView& v, bool now, bool next_step, cudaStream_t st) {
  mark_rebuild_kernel<<<1, 1, 0, st>>>(v.sc, now ? 1 : 0, next_step ? 1 : 0);
}

void launch_sort(const DevView& v, cudaStream_t st) {
  const Scratch& S = v.S;
  const int ncells = v.total_cells;
  const int xsub = v.o.xsub;
  const int nbins = ncells * xsub;
  const int len = nbins + 2;
  int* sstart = xsub > 1 ? S.sstart : S.start;  // one slab per cell: the slab starts are the cell starts
  cudaMemsetAsync(S.count, 0, sizeof(int) * (size_t)len, st);
  bin_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(v, v.alive, S.key, S.count, v.sc, v.o.dim, xsub);
  const int nb = (len + 1023) / 1024;
  scan_blocks<<<nb, 1024, 0, st>>>(S.count, sstart, S.block_sums, len, v.sc);
  scan_sums<<<1, 1024, 0, st>>>(S.block_sums, nb, sstart + len, v.sc);
  scan_add<<<nb, 1024, 0, st>>>(sstart, S.block_sums, len, v.sc);
  cudaMemsetAsync(S.count, 0, sizeof(int) * (size_t)len, st);
  scatter_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(S.key, sstart, S.count, S.tmp_perm, v.sc);
  rank_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(S.key, sstart, S.tmp_perm, v, S.perm, v.sc, nbins);
  reorder_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(v, S.perm, S.key, sstart, S.cellid, v.alive, v.sc, nbins, xsub,
                                                    v.o.has_solid, v.o.dyn_mu);
  if (v.o.has_solid) reorder_tensors_kernel<<<grid_for(v.ncap), kBT, 0, st>>>(v, S.perm, sstart, v.sc, nbins);
  finish_sort_kernel<<<1, 1, 0, st>>>(sstart, v.sc, nbins);
  cell_starts_kernel<<<grid_for(ncells + 3), kBT, 0, st>>>(sstart, S.start, ncells, xsub, v.sc, S.tmp_perm, v.ncap);
}

}  // namespace psph

namespace psph {

// Exclusive prefix of in[0..len) into out[0..len], out[len] = total, using
// block_sums (>= ceil(len/1024) entries) as scratch. Used by the pair export
// that takes its scratch from caller-owned or static device memory.
void launch_exclusive_scan(const int* in, int* out, int len, int* block_sums, cudaStream_t st) {
  const int nb = (len + 1023) / 1024 > 0 ? (len + 1023) / 1024 : 1;
  scan_blocks<<<nb, 1024, 0, st>>>(in, out, block_sums, len, nullptr);
  scan_sums<<<1, 1024, 0, st>>>(block_sums, nb, out + len, nullptr);
  scan_add<<<nb, 1024, 0, st>>>(out, block_sums, len, nullptr);
}

}  // namespace psph
