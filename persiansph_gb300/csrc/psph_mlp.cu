// Learned eddy-viscosity closure: a 6 -> 64 -> 64 -> 64 -> 1 SiLU network.
//
//  * closure_kernel (inside the step) and infer_tc_kernel run the three hidden
//    layers on the 5th-generation tensor cores: one CTA of 128 threads per
//    128-particle tile, BF16 activations written by the threads into a
//    128-byte-swizzled shared-memory tile, BF16 weights brought in once per CTA
//    by a TMA bulk copy, tcgen05.mma issued by one thread with the FP32
//    accumulator in tensor memory, tcgen05.ld back to registers (thread t owns
//    row t) for bias + SiLU; the 64 -> 1 output layer runs on the CUDA cores.
//  * Training runs on the tensor cores too (train_tc_kernel): per 128-sample
//    tile the forward pass (three MMAs, pre-activations kept for the backward
//    pass), the loss gradient, the backward deltas of the hidden layers as MMAs
//    against transposed weight images (BF16 deltas, FP32 accumulation), and the
//    gradients of W2 and W3 as MMAs with the samples along K (deltas^T times
//    activations), accumulated in tensor memory over the CTA's tiles. The small
//    parameters (W1, biases, output layer) are summed on the CUDA cores; every
//    sum has a fixed order (per-CTA partials, then one reduction) and Adam
//    follows, so a training run is deterministic. Straight-through gradients
//    through the BF16 roundings of weights, activations and deltas.
// Every wait on a tensor-core or copy completion is bounded (1 s); a wait that
// gives up sets ST_CLOSURE_TIMEOUT (or an error status) and the kernel returns
// after freeing its tensor memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "psph_device.cuh"
#include "psph_mlp.cuh"

using namespace psph;

namespace {

// ---------------------------------------------------------------------------
// scalar helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.f + z * (1.f - s));
}
// SiLU of the tensor-core inference epilogues: hardware exp2 and reciprocal
// approximations (relative error ~1e-6, far below the BF16 rounding of the
// activations that follows). z is clamped at -80 so 1 + exp(-z) stays a
// normal float, where the approximate division is defined.
__device__ __forceinline__ float silu_fast(float z) { return z * __fdividef(1.f, 1.f + __expf(-fmaxf(z, -80.f))); }
// SiLU for the activations that are rounded to BF16 right after (hidden layers
// 1 and 2): z sigmoid(z) = z/2 (1 + tanh(z/2)) with the hardware tanh
// approximation (relative error ~2^-11, below the BF16 rounding of 2^-9), one
// special-function operation instead of two.
__device__ __forceinline__ float silu_tanh(float z) {
  const float h = 0.5f * z;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}
__device__ __forceinline__ float softplus(float z) { return z > 20.f ? z : log1pf(expf(z)); }

// ---------------------------------------------------------------------------
// tensor-core, mbarrier and bulk-copy primitives (inline PTX, sm_100 family)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase with the given parity to complete, giving up after limit_ns.
__device__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > limit_ns) return false;
  }
  return true;
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> shared (TMA), completion counted on the mbarrier.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (start address, LBO, SBO, version 1, layout 2).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major,
// N = 64, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kMlpH >> 3) << 17) |
                            ((uint32_t)(kMlpTile >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t addr, float* z) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(addr)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) z[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

// ---------------------------------------------------------------------------
// tensor-core tile forward, shared by the closure and the standalone inference
// ---------------------------------------------------------------------------
constexpr int kTcThreads = kMlpTile;           // thread t owns tile row t
constexpr int kSmA = 0;                         // A tile: 128 rows x 128 B
constexpr int kSmW = kSmA + kMlpTile * 128;     // W1..W3 images, 8 KB each
constexpr int kSmPad = kSmW + 3 * kImgBytes;    // 8 KB of slack after the operands
constexpr int kSmF = kSmPad + 8192;             // floats: b1 b2 b3 w4 (256) + b4 + norm (24)
constexpr int kSmFloats = 4 * kMlpH + 4 + 4 * kMlpIn;
constexpr int kTcSmemBytes = kSmF + kSmFloats * 4 + 1024;  // + alignment slack

struct TcCtx {
  uint8_t* a;
  uint8_t* w;        // three images back to back
  float* f;          // b1, b2, b3, w4, b4(+3 pad), mean, inv_std, lo, hi
  uint64_t* bar_mma;
  int* err;
  uint32_t taddr;
  uint32_t phase;
};

__device__ __forceinline__ const float* tc_b(const TcCtx& t, int l) { return t.f + l * kMlpH; }

// Loads the image into shared memory (bulk copy for the operand images) and
// allocates the 64 accumulator columns. All threads call it.
__device__ bool tc_setup(TcCtx& t, uint8_t* smem_raw, const MlpImage* img, uint64_t* bars, uint32_t* slot, int* err) {
  const int tid = threadIdx.x;
  const uint32_t base = smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (base & 1023)) & 1023);  // 1024-byte aligned for the swizzle atoms
  t.a = sm + kSmA;
  t.w = sm + kSmW;
  t.f = reinterpret_cast<float*>(sm + kSmF);
  t.bar_mma = &bars[1];
  t.err = err;
  t.phase = 0;
  if (tid == 0) {
    *err = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  // biases, output layer and normalisation: plain loads
  const float* src = img->b1;
  for (int k = tid; k < kSmFloats; k += blockDim.x) t.f[k] = src[k];
  if (tid < 32) tmem_alloc(slot, kMlpH);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  t.taddr = *slot;
  if (tid == 0) {
    mbar_expect_tx(&bars[0], 3 * kImgBytes);
    bulk_g2s(t.w, img->w1, kImgBytes, &bars[0]);
    bulk_g2s(t.w + kImgBytes, img->w2, kImgBytes, &bars[0]);
    bulk_g2s(t.w + 2 * kImgBytes, img->w3, kImgBytes, &bars[0]);
    if (!mbar_wait_bounded(&bars[0], 0, 1000000000ull)) *err = 1;
  }
  __syncthreads();
  return *err == 0;
}

__device__ void tc_teardown(TcCtx& t) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(t.taddr, kMlpH);
}

// Row r of the A tile from 64 values (BF16, swizzled).
__device__ __forceinline__ void store_row64(uint8_t* a, int r, const float* x) {
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    uint4 q;
    q.x = pack_bf16(x[8 * c + 0], x[8 * c + 1]);
    q.y = pack_bf16(x[8 * c + 2], x[8 * c + 3]);
    q.z = pack_bf16(x[8 * c + 4], x[8 * c + 5]);
    q.w = pack_bf16(x[8 * c + 6], x[8 * c + 7]);
    *reinterpret_cast<uint4*>(a + sw128_offset(r, 8 * c)) = q;
  }
}

// One layer: D = A W^T over ksteps K-steps of 16, then each thread reads its
// row of D. Returns false when the completion wait gave up.
__device__ bool tc_layer(TcCtx& t, int layer, int ksteps, float* z) {
  proxy_fence_smem();  // the threads' A writes become visible to the tensor core
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    const uint64_t ad = sw128_desc(smem_u32(t.a));
    const uint64_t bd = sw128_desc(smem_u32(t.w + layer * kImgBytes));
    for (int k = 0; k < ksteps; ++k) mma_bf16(t.taddr, ad + 2 * k, bd + 2 * k, k > 0 ? 1u : 0u);
    mma_commit(t.bar_mma);
    if (!mbar_wait_bounded(t.bar_mma, t.phase, 1000000000ull)) *t.err = 1;
  }
  t.phase ^= 1u;
  __syncthreads();
  tc_fence_after();
  if (*t.err) return false;
  const uint32_t lane_addr = t.taddr + ((uint32_t)(threadIdx.x & ~31) << 16);
#pragma unroll
  for (int j = 0; j < 4; ++j) tmem_ld16(lane_addr + 16 * j, z + 16 * j);
  tmem_wait_ld();
  return true;
}

// Network output z4 for this thread's row; u = standardised features.
__device__ bool tc_forward(TcCtx& t, const float* u, float* out) {
  const int r = threadIdx.x;
  float z[kMlpH];
  {
    float x[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) x[k] = (k < kMlpIn) ? u[k] : 0.f;
    uint4 q0, q1;
    q0.x = pack_bf16(x[0], x[1]); q0.y = pack_bf16(x[2], x[3]); q0.z = pack_bf16(x[4], x[5]); q0.w = pack_bf16(x[6], x[7]);
    q1.x = pack_bf16(x[8], x[9]); q1.y = pack_bf16(x[10], x[11]); q1.z = pack_bf16(x[12], x[13]); q1.w = pack_bf16(x[14], x[15]);
    *reinterpret_cast<uint4*>(t.a + sw128_offset(r, 0)) = q0;
    *reinterpret_cast<uint4*>(t.a + sw128_offset(r, 8)) = q1;
  }
  if (!tc_layer(t, 0, 1, z)) return false;
  const float* b1 = tc_b(t, 0);
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) z[k] = silu_tanh(z[k] + b1[k]);
  store_row64(t.a, r, z);
  if (!tc_layer(t, 1, kMlpH / 16, z)) return false;
  const float* b2 = tc_b(t, 1);
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) z[k] = silu_tanh(z[k] + b2[k]);
  store_row64(t.a, r, z);
  if (!tc_layer(t, 2, kMlpH / 16, z)) return false;
  const float* b3 = tc_b(t, 2);
  const float* w4 = tc_b(t, 3);
  float o = t.f[4 * kMlpH];
#pragma unroll
  for (int k = 0; k < kMlpH; ++k) o += w4[k] * silu_fast(z[k] + b3[k]);
  *out = o;
  return true;
}

__device__ __forceinline__ const float* tc_norm(const TcCtx& t) { return t.f + 4 * kMlpH + 4; }

// ---------------------------------------------------------------------------
// closure inside the step
// ---------------------------------------------------------------------------
// F32: the FP32C form, whose pair kernel leaves the shear-rate features in
// FP32 (no FP64 arithmetic here); otherwise the features come from the FP64
// strain-rate sums with FP64 contractions.
template <int DIM, bool F32>
__global__ void __launch_bounds__(kTcThreads) closure_kernel(DevView v) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t slot;
  __shared__ int err;
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  TcCtx t;
  const bool ok = tc_setup(t, smem_raw, static_cast<const MlpImage*>(v.mlp), bars, &slot, &err);
  const int n = sc->n;
  const int ntiles = (n + kMlpTile - 1) / kMlpTile;
  const Persist& P = cur_persist(v);
  const float* nm = tc_norm(t);
  const float* mean = nm;
  const float* inv_std = nm + kMlpIn;
  const float* lo = nm + 2 * kMlpIn;
  const float* hi = nm + 3 * kMlpIn;
  unsigned long long n_eval = 0, n_fb = 0;
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    const int s = tile * kMlpTile + threadIdx.x;
    bool act = false;
    float f[kMlpIn] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    double shear = 0.0, h = 0.0;
    if (s < n && F32) {
      const PClass32& C = v.cls32[P.cls[s]];
      act = (C.flags & CF_FREE) && C.material == 1 && (C.flags & CF_LES) && !v.inst[C.inst].stop;
      float sh32 = 0.f;
      if (act) {
        sh32 = v.S.cshear[s];
        const float tscale = C.cs > 0.f ? C.h / C.cs : 1.f;
        f[0] = logf(fmaxf(sh32 * tscale, 1e-12f));
        f[1] = v.S.cr3[s];
        f[2] = logf(fmaxf(v.S.cvort[s] * tscale, 1e-12f));
        f[3] = v.S.D32[s].w / C.rho0;
        f[4] = C.h_over_dx;
        f[5] = v.S.cnnb[s];
      }
      shear = sh32;
      h = C.h;
      float* fo = v.S.cfeat + (size_t)kMlpIn * s;
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) fo[k] = f[k];
    } else if (s < n) {
      const PClass& C = v.cls[P.cls[s]];
      act = C.is_free && C.material == 1 && C.les && !v.inst[C.inst].stop;
      if (act) {
        const double* S = v.S.strain_rate + 9 * (size_t)s;
        // same contraction as Mat1's ShearRate (Source/Particle.cpp:151-153)
        const double temp =
            (S[0] * S[0] + 2.0 * S[1] * S[3] + 2.0 * S[2] * S[6] + S[4] * S[4] + 2.0 * S[5] * S[7] + S[8] * S[8]);
        shear = sqrt(0.5 * temp);
        const double det = S[0] * (S[4] * S[8] - S[5] * S[7]) - S[1] * (S[3] * S[8] - S[5] * S[6]) +
                           S[2] * (S[3] * S[7] - S[4] * S[6]);
        h = C.h;
        // rates in units of the acoustic rate Cs/h (the lattice-independent
        // form: the same flow resolved at another dx keeps its features)
        const double tscale = C.cs > 0.0 ? C.h / C.cs : 1.0;
        f[0] = logf(fmaxf((float)(shear * tscale), 1e-12f));
        f[1] = temp > 0.0 ? (float)(det / (temp * sqrt(temp))) : 0.f;
        f[2] = logf(fmaxf(v.S.cvort[s] * (float)tscale, 1e-12f));
        f[3] = (float)(P.X4[s].w / C.rho0);
        f[4] = (float)(C.h / v.o.closure_dx);
        f[5] = v.S.cnnb[s];
      }
      float* fo = v.S.cfeat + (size_t)kMlpIn * s;
#pragma unroll
      for (int k = 0; k < kMlpIn; ++k) fo[k] = f[k];
    }
    // A shear rate or vorticity below the trained range is fluid at rest: the
    // eddy viscosity c h^2 ShearRate vanishes with it whatever c is, so the
    // two rate features are raised to the range's floor instead of falling
    // back; anything else outside [lo, hi] takes the Smagorinsky term.
    f[0] = fmaxf(f[0], lo[0]);
    f[2] = fmaxf(f[2], lo[2]);
    bool in_range = act;
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) in_range = in_range && f[k] >= lo[k] && f[k] <= hi[k];
    float u[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) u[k] = in_range ? (f[k] - mean[k]) * inv_std[k] : 0.f;
    float z4 = 0.f;
    if (!tc_forward(t, u, &z4)) break;
    if (act) {
      if (F32) v.S.nut[s] = in_range ? (double)(softplus(z4) * (float)h * (float)h * (float)shear) : -1.0;
      else v.S.nut[s] = in_range ? (double)softplus(z4) * h * h * shear : -1.0;
    }
    n_eval += act ? 1 : 0;
    n_fb += (act && !in_range) ? 1 : 0;
  }
  // per-CTA totals (order-independent integer sums)
  for (int off = 16; off > 0; off >>= 1) {
    n_eval += __shfl_down_sync(0xffffffffu, n_eval, off);
    n_fb += __shfl_down_sync(0xffffffffu, n_fb, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (n_eval) atomicAdd(&v.sc->closure_eval, n_eval);
    if (n_fb) atomicAdd(&v.sc->closure_fallback, n_fb);
  }
  if (err && threadIdx.x == 0) atomicOr(&v.sc->status, ST_CLOSURE_TIMEOUT);
  tc_teardown(t);
}

// ---------------------------------------------------------------------------
// standalone inference (tensor cores / CUDA cores)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTcThreads) infer_tc_kernel(const MlpImage* img, const float* x, int n, float* c,
                                                              int* status) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t slot;
  __shared__ int err;
  TcCtx t;
  const bool ok = tc_setup(t, smem_raw, img, bars, &slot, &err);
  const float* nm = tc_norm(t);
  const int ntiles = (n + kMlpTile - 1) / kMlpTile;
  for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    const int s = tile * kMlpTile + threadIdx.x;
    float u[kMlpIn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) u[k] = (s < n) ? (x[(size_t)kMlpIn * s + k] - nm[k]) * nm[kMlpIn + k] : 0.f;
    float z4 = 0.f;
    if (!tc_forward(t, u, &z4)) break;
    if (s < n) c[s] = softplus(z4);
  }
  if (err && threadIdx.x == 0) atomicExch(status, 1);
  tc_teardown(t);
}

// FP32 forward of one sample with the BF16 roundings of the tensor-core path;
// stores the pre-activations when z1 != nullptr (training).
__device__ float cc_forward(const float* __restrict__ p, const float* u_in, float* u_out, float* z1, float* z2,
                            float* z3) {
  float u[kMlpIn];
#pragma unroll
  for (int k = 0; k < kMlpIn; ++k) u[k] = bf16r(u_in[k]);
  if (u_out)
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) u_out[k] = u[k];
  float a1[kMlpH], a2[kMlpH];
#pragma unroll
  for (int nn = 0; nn < kMlpH; ++nn) {
    float z = p[kOB1 + nn];
#pragma unroll
    for (int k = 0; k < kMlpIn; ++k) z += bf16r(p[kOW1 + nn * kMlpIn + k]) * u[k];
    if (z1) z1[nn] = z;
    a1[nn] = bf16r(silu(z));
  }
#pragma unroll 4
  for (int nn = 0; nn < kMlpH; ++nn) {
    float z = p[kOB2 + nn];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z += bf16r(p[kOW2 + nn * kMlpH + k]) * a1[k];
    if (z2) z2[nn] = z;
    a2[nn] = bf16r(silu(z));
  }
  float o = p[kOB4];
#pragma unroll 4
  for (int nn = 0; nn < kMlpH; ++nn) {
    float z = p[kOB3 + nn];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z += bf16r(p[kOW3 + nn * kMlpH + k]) * a2[k];
    if (z3) z3[nn] = z;
    o += p[kOW4 + nn] * silu(z);
  }
  return o;
}

__global__ void infer_cc_kernel(const float* __restrict__ params, const float* __restrict__ norm, const float* x,
                                int n, float* c) {
  __shared__ float p[kNParams];
  for (int k = threadIdx.x; k < kNParams; k += blockDim.x) p[k] = params[k];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float u[kMlpIn];
  for (int k = 0; k < kMlpIn; ++k) u[k] = (x[(size_t)kMlpIn * s + k] - norm[k]) * norm[kMlpIn + k];
  c[s] = softplus(cc_forward(p, u, nullptr, nullptr, nullptr, nullptr));
}

// ---------------------------------------------------------------------------
// training: the parameters the tensor cores do not take (CUDA cores, FP32)
// ---------------------------------------------------------------------------
constexpr int kTrainThreads = 128;

// Gradient of W1, the biases and the output layer summed over one chunk of
// samples: part[chunk][param] (W2 and W3 come from the tensor cores). Threads
// of a warp take consecutive parameters, so the activation reads of a weight
// row are contiguous.
__global__ void train_wgrad_kernel(const float* __restrict__ U, const float* __restrict__ Z1,
                                   const float* __restrict__ Z2, const float* __restrict__ Z3,
                                   const float* __restrict__ G4, const float* __restrict__ D1,
                                   const float* __restrict__ D2, const float* __restrict__ D3, int B, int chunk,
                                   float* part) {
  const int pidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (pidx >= kNParams) return;
  const int b0 = blockIdx.y * chunk, b1 = min(B, b0 + chunk);
  float acc = 0.f;
  if (pidx < kOB1) {
    const int nn = pidx / kMlpIn, k = pidx % kMlpIn;
    for (int b = b0; b < b1; ++b) acc += D1[(size_t)kMlpH * b + nn] * U[(size_t)8 * b + k];
  } else if (pidx < kOW2) {
    const int nn = pidx - kOB1;
    for (int b = b0; b < b1; ++b) acc += D1[(size_t)kMlpH * b + nn];
  } else if (pidx < kOB2) {  // W2: the tensor-core partials
  } else if (pidx < kOW3) {
    const int nn = pidx - kOB2;
    for (int b = b0; b < b1; ++b) acc += D2[(size_t)kMlpH * b + nn];
  } else if (pidx < kOB3) {  // W3: the tensor-core partials
  } else if (pidx < kOW4) {
    const int nn = pidx - kOB3;
    for (int b = b0; b < b1; ++b) acc += D3[(size_t)kMlpH * b + nn];
  } else if (pidx < kOB4) {
    const int k = pidx - kOW4;
    for (int b = b0; b < b1; ++b) acc += G4[b] * silu(Z3[(size_t)kMlpH * b + k]);
  } else {
    for (int b = b0; b < b1; ++b) acc += G4[b];
  }
  part[(size_t)blockIdx.y * kNParams + pidx] = acc;
}

// Sums the per-chunk partials of the CUDA-core parameters and, for W2 and W3,
// the per-CTA tensor-core partials (mma[cta][0] = dW3, mma[cta][1] = dW2, row =
// output unit, column = input unit), each in a fixed order.
__global__ void train_reduce_kernel(const float* __restrict__ part, int nchunks, const float* __restrict__ mma,
                                    int nctas, float* grad) {
  const int pidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (pidx >= kNParams) return;
  float s = 0.f;
  const bool w2 = pidx >= kOW2 && pidx < kOB2, w3 = pidx >= kOW3 && pidx < kOB3;
  if (w2 || w3) {
    const int q = w2 ? pidx - kOW2 : pidx - kOW3;
    for (int c = 0; c < nctas; ++c) s += mma[((size_t)c * 2 + (w2 ? 1 : 0)) * kMlpH * kMlpH + q];
  } else {
    for (int c = 0; c < nchunks; ++c) s += part[(size_t)c * kNParams + pidx];
  }
  grad[pidx] = s;
}

// ---------------------------------------------------------------------------
// training on the tensor cores
// ---------------------------------------------------------------------------
// The operand images of one optimizer step, built on the device from the FP32
// master parameters: W1 (K padded to 16), W2 and W3 (row = output unit, K =
// input unit) for the forward pass; W2^T and W3^T (row = input unit, K =
// output unit) for the backward pass.
struct TrainImages {
  uint8_t w[5][kImgBytes];  // W1, W2, W3, W2^T, W3^T
};

__global__ void train_images_kernel(const float* __restrict__ p, TrainImages* img) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 5 * kMlpH * kMlpH) return;
  const int im = idx / (kMlpH * kMlpH), r = (idx / kMlpH) % kMlpH, k = idx % kMlpH;
  float w;
  switch (im) {
    case 0: w = k < kMlpIn ? p[kOW1 + r * kMlpIn + k] : 0.f; break;
    case 1: w = p[kOW2 + r * kMlpH + k]; break;
    case 2: w = p[kOW3 + r * kMlpH + k]; break;
    case 3: w = p[kOW2 + k * kMlpH + r]; break;
    default: w = p[kOW3 + k * kMlpH + r]; break;
  }
  *reinterpret_cast<__nv_bfloat16*>(img->w[im] + sw128_offset(r, k)) = __float2bfloat16_rn(w);
}

// shared memory of train_tc_kernel (offsets from a 1024-byte aligned base)
constexpr int kTrA = 0;                            // A tile: 128 rows x 64 BF16 (16 KB)
constexpr int kTrW = kTrA + kMlpTile * 128;        // the five operand images (40 KB)
constexpr int kTrDT = kTrW + 5 * kImgBytes;        // deltas^T of layers 3 and 2: 2 x (2 x [128 x 64]) (64 KB)
constexpr int kTrAT = kTrDT + 4 * kMlpTile * 128;  // activations^T a2, a1: 2 x (2 x [64 x 64]) (32 KB)
constexpr int kTrF = kTrAT + 4 * kImgBytes;        // b1 b2 b3 w4 b4 (+3) and the normalisation
constexpr int kTrSmemBytes = kTrF + kSmFloats * 4 + 1024;
constexpr int kTrCols = 256;                       // TMEM: layer accumulator 0-63, dW3 64-127, dW2 128-191

// D[128 x 64] (+)= A[128 x 16 ksteps] B[64 x 16 ksteps]^T, A and B K-major in
// 64-column sub-tiles of a_stride / b_stride bytes (the caller commits).
__device__ __forceinline__ void tc_mma_chain(uint32_t tmem_d, const uint8_t* a, int a_stride, const uint8_t* b,
                                             int b_stride, int ksteps, bool accumulate) {
  for (int k = 0; k < ksteps; ++k) {
    const uint64_t ad = sw128_desc(smem_u32(a + (k >> 2) * a_stride)) + 2 * (k & 3);
    const uint64_t bd = sw128_desc(smem_u32(b + (k >> 2) * b_stride)) + 2 * (k & 3);
    mma_bf16(tmem_d, ad, bd, (accumulate || k > 0) ? 1u : 0u);
  }
}

// Every thread: its writes to the operand tiles become visible to the tensor
// core, then thread 0 runs the MMAs and waits; afterwards the accumulator is
// readable. Returns false when the wait gave up.
template <class F>
__device__ bool tc_sync_mma(uint64_t* bar, uint32_t& phase, int* err, F&& issue) {
  proxy_fence_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    issue();
    mma_commit(bar);  // one arrival for everything issued
    if (!mbar_wait_bounded(bar, phase, 1000000000ull)) *err = 1;
  }
  phase ^= 1u;
  __syncthreads();
  tc_fence_after();
  return *err == 0;
}

__device__ __forceinline__ void tmem_row64(uint32_t taddr, int col, float* z) {
  const uint32_t a = taddr + ((uint32_t)(threadIdx.x & ~31) << 16) + (uint32_t)col;
#pragma unroll
  for (int j = 0; j < 4; ++j) tmem_ld16(a + 16 * j, z + 16 * j);
  tmem_wait_ld();
}

// column c of a transposed operand ([rows] x 128 samples, two 64-wide
// sub-tiles of sub_bytes): 64 values of this thread's sample
__device__ __forceinline__ void store_col64(uint8_t* t, int sub_bytes, int c, const float* x) {
  uint8_t* base = t + (c >> 6) * sub_bytes;
  const int k = c & 63;
#pragma unroll
  for (int r = 0; r < kMlpH; ++r)
    *reinterpret_cast<__nv_bfloat16*>(base + sw128_offset(r, k)) = __float2bfloat16_rn(x[r]);
}

// One CTA of 128 threads per tile of 128 samples (thread t = sample t of the
// tile), looping over tiles; writes the activations and deltas the CUDA-core
// gradients need (U, Z1..Z4, G4, D1..D3), the loss partial of each tile, and
// its tensor-core partials of dW3 and dW2 (mma[cta][2][64][64]).
__global__ void __launch_bounds__(kTcThreads) train_tc_kernel(
    const TrainImages* __restrict__ img, const float* __restrict__ params, const float* __restrict__ norm,
    const float* __restrict__ X, const float* __restrict__ Y, const float* __restrict__ W, const int* __restrict__ idx,
    int B, float* U, float* Z1, float* Z2, float* Z3, float* Z4, float* G4, float* D1, float* D2, float* D3,
    double* loss_part, float* mma, int* status) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t slot;
  __shared__ int err;
  __shared__ double lred[kTcThreads / 32];
  const int tid = threadIdx.x;
  const uint32_t sbase = smem_u32(smem_raw);
  uint8_t* sm = smem_raw + ((1024 - (sbase & 1023)) & 1023);
  uint8_t* A = sm + kTrA;
  uint8_t* Wi = sm + kTrW;
  uint8_t* DT = sm + kTrDT;  // [2 layers][2 sub-tiles][128 rows x 128 B]
  uint8_t* AT = sm + kTrAT;  // [2 layers][2 sub-tiles][64 rows x 128 B]
  float* f = reinterpret_cast<float*>(sm + kTrF);
  constexpr int kDsub = kMlpTile * 128, kAsub = kImgBytes;
  uint8_t* dt3 = DT;
  uint8_t* dt2 = DT + 2 * kDsub;
  uint8_t* at2 = AT;
  uint8_t* at1 = AT + 2 * kAsub;
  if (tid == 0) {
    err = 0;
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  // biases, output layer and normalisation; the delta tiles' rows 64-127 stay
  // zero (M is 128, the layers have 64 units)
  for (int k = tid; k < 4 * kMlpH; k += blockDim.x) {
    const int seg = k / kMlpH, e = k % kMlpH;
    f[k] = params[(seg == 0 ? kOB1 : seg == 1 ? kOB2 : seg == 2 ? kOB3 : kOW4) + e];
  }
  if (tid == 0) f[4 * kMlpH] = params[kOB4];
  for (int k = tid; k < 2 * kMlpIn; k += blockDim.x) f[4 * kMlpH + 4 + k] = norm[k];
  for (int k = tid; k < 4 * kDsub / 16; k += blockDim.x) reinterpret_cast<uint4*>(DT)[k] = make_uint4(0, 0, 0, 0);
  if (tid < 32) tmem_alloc(&slot, kTrCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t taddr = slot;
  if (tid == 0) {
    mbar_expect_tx(&bars[0], 5 * kImgBytes);
    bulk_g2s(Wi, img->w[0], 5 * kImgBytes, &bars[0]);
    if (!mbar_wait_bounded(&bars[0], 0, 1000000000ull)) err = 1;
  }
  __syncthreads();
  uint32_t phase = 0;
  const float* b1 = f;
  const float* b2 = f + kMlpH;
  const float* b3 = f + 2 * kMlpH;
  const float* w4 = f + 3 * kMlpH;
  const float* mean = f + 4 * kMlpH + 4;
  const float* inv_std = mean + kMlpIn;
  const int ntiles = (B + kMlpTile - 1) / kMlpTile;
  bool first = true;
  float z[kMlpH], d[kMlpH];
  for (int tile = blockIdx.x; tile < ntiles && !err; tile += gridDim.x) {
    const int b = tile * kMlpTile + tid;
    const bool valid = b < B;
    const int row = valid ? (idx ? idx[b] : b) : 0;
    // layer 1: standardised features, BF16, K padded to 16
    float u[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) u[k] = (valid && k < kMlpIn) ? bf16r((X[(size_t)kMlpIn * row + k] - mean[k]) * inv_std[k]) : 0.f;
    {
      uint4 q0, q1;
      q0.x = pack_bf16(u[0], u[1]); q0.y = pack_bf16(u[2], u[3]); q0.z = pack_bf16(u[4], u[5]); q0.w = pack_bf16(u[6], u[7]);
      q1.x = pack_bf16(u[8], u[9]); q1.y = pack_bf16(u[10], u[11]); q1.z = pack_bf16(u[12], u[13]); q1.w = pack_bf16(u[14], u[15]);
      *reinterpret_cast<uint4*>(A + sw128_offset(tid, 0)) = q0;
      *reinterpret_cast<uint4*>(A + sw128_offset(tid, 8)) = q1;
    }
    if (!tc_sync_mma(&bars[1], phase, &err, [&] { tc_mma_chain(taddr, A, 0, Wi, 0, 1, false); })) break;
    tmem_row64(taddr, 0, z);
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z[k] += b1[k];
    if (valid) {
      for (int k = 0; k < kMlpH; ++k) Z1[(size_t)kMlpH * b + k] = z[k];
      for (int k = 0; k < 8; ++k) U[(size_t)8 * b + k] = k < kMlpIn ? u[k] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z[k] = bf16r(silu(z[k]));
    store_row64(A, tid, z);
    store_col64(at1, kAsub, tid, z);
    // layer 2
    if (!tc_sync_mma(&bars[1], phase, &err, [&] { tc_mma_chain(taddr, A, 0, Wi + kImgBytes, 0, 4, false); }))
      break;
    tmem_row64(taddr, 0, z);
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z[k] += b2[k];
    if (valid)
      for (int k = 0; k < kMlpH; ++k) Z2[(size_t)kMlpH * b + k] = z[k];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) z[k] = bf16r(silu(z[k]));
    store_row64(A, tid, z);
    store_col64(at2, kAsub, tid, z);
    // layer 3 and the output
    if (!tc_sync_mma(&bars[1], phase, &err, [&] { tc_mma_chain(taddr, A, 0, Wi + 2 * kImgBytes, 0, 4, false); }))
      break;
    tmem_row64(taddr, 0, z);
    float o = f[4 * kMlpH];
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) {
      z[k] += b3[k];
      o += w4[k] * silu(z[k]);
    }
    // loss and its gradient (mean over the minibatch)
    double lp = 0.0;
    float g = 0.f;
    if (valid) {
      const float y = Y[row], w = W ? W[row] : 1.f;
      const float e = softplus(o) - y;
      g = 2.f * w * e * sigm(o) / (float)B;
      lp = (double)w * (double)e * (double)e;
      Z4[b] = o;
      G4[b] = g;
      for (int k = 0; k < kMlpH; ++k) Z3[(size_t)kMlpH * b + k] = z[k];
    }
    for (int off = 16; off > 0; off >>= 1) lp += __shfl_down_sync(0xffffffffu, lp, off);
    if ((tid & 31) == 0) lred[tid >> 5] = lp;
    // delta of layer 3
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) d[k] = g * w4[k] * dsilu(z[k]);
    if (valid)
      for (int k = 0; k < kMlpH; ++k) D3[(size_t)kMlpH * b + k] = d[k];
    store_row64(A, tid, d);
    store_col64(dt3, kDsub, tid, d);
    // delta of layer 2: (d3 W3) o silu'(z2)
    if (!tc_sync_mma(&bars[1], phase, &err, [&] { tc_mma_chain(taddr, A, 0, Wi + 4 * kImgBytes, 0, 4, false); }))
      break;
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < kTcThreads / 32; ++w) t += lred[w];
      loss_part[tile] = t;
    }
    tmem_row64(taddr, 0, d);
#pragma unroll
    for (int k = 0; k < kMlpH; ++k) d[k] *= dsilu(valid ? Z2[(size_t)kMlpH * b + k] : 0.f);
    if (valid)
      for (int k = 0; k < kMlpH; ++k) D2[(size_t)kMlpH * b + k] = d[k];
    store_row64(A, tid, d);
    store_col64(dt2, kDsub, tid, d);
    // delta of layer 1: (d2 W2) o silu'(z1)
    if (!tc_sync_mma(&bars[1], phase, &err, [&] { tc_mma_chain(taddr, A, 0, Wi + 3 * kImgBytes, 0, 4, false); }))
      break;
    tmem_row64(taddr, 0, d);
    if (valid)
      for (int k = 0; k < kMlpH; ++k) D1[(size_t)kMlpH * b + k] = d[k] * dsilu(Z1[(size_t)kMlpH * b + k]);
    // dW3 += d3^T a2 and dW2 += d2^T a1 over this tile's samples (K = 128)
    const bool acc = !first;
    if (!tc_sync_mma(&bars[1], phase, &err, [&] {
          tc_mma_chain(taddr + 64, dt3, kDsub, at2, kAsub, 8, acc);
          tc_mma_chain(taddr + 128, dt2, kDsub, at1, kAsub, 8, acc);
        }))
      break;
    first = false;
  }
  // this CTA's dW3 / dW2 rows (TMEM lanes 0-63 = output units)
  if (!err && !first && tid < kMlpH) {
    float* out = mma + (size_t)blockIdx.x * 2 * kMlpH * kMlpH;
    tmem_row64(taddr, 64, z);
    for (int k = 0; k < kMlpH; ++k) out[(size_t)tid * kMlpH + k] = z[k];
    tmem_row64(taddr, 128, z);
    for (int k = 0; k < kMlpH; ++k) out[(size_t)(kMlpH + tid) * kMlpH + k] = z[k];
  } else if (!err && first && tid < kMlpH) {  // no tile: zero partials
    float* out = mma + (size_t)blockIdx.x * 2 * kMlpH * kMlpH;
    for (int k = 0; k < 2 * kMlpH; ++k) out[(size_t)(k / kMlpH * kMlpH + tid) * kMlpH + k % kMlpH] = 0.f;
  }
  if (err && tid == 0) atomicExch(status, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (tid < 32) tmem_dealloc(taddr, kTrCols);
}

__global__ void adam_kernel(float* params, const float* grad, float* m, float* v, float lr, float b1, float b2,
                            float c1, float c2, float eps) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kNParams) return;
  const float g = grad[k];
  const float mk = b1 * m[k] + (1.f - b1) * g;
  const float vk = b2 * v[k] + (1.f - b2) * g * g;
  m[k] = mk;
  v[k] = vk;
  params[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
uint16_t bf16_bits(float f) {  // round to nearest even
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

void put_operand(uint8_t* img, const float* W, int rows, int cols) {  // W[rows][cols] -> swizzled K-major
  std::memset(img, 0, kImgBytes);
  for (int r = 0; r < rows; ++r)
    for (int k = 0; k < cols; ++k) {
      const uint16_t b = bf16_bits(W[r * cols + k]);
      std::memcpy(img + sw128_offset(r, k), &b, 2);
    }
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 148;
  }
  return n;
}

bool tr_attr_set = false;
cudaError_t ensure_train_attrs() {
  if (tr_attr_set) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmemBytes);
  if (e == cudaSuccess) tr_attr_set = true;
  return e;
}

bool tc_attr_set = false;
cudaError_t ensure_tc_attrs() {
  if (tc_attr_set) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(closure_kernel<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(closure_kernel<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(closure_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(closure_kernel<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  if (e == cudaSuccess) tc_attr_set = true;
  return e;
}

}  // namespace

namespace psph {
void launch_closure(const DevView& v, cudaStream_t st) {
  if (ensure_tc_attrs() != cudaSuccess) return;  // the launch below then reports the error
  const int ntiles = (v.ncap + kMlpTile - 1) / kMlpTile;
  // four CTAs per SM (128 registers x 128 threads, ~52 KB shared memory and 64
  // TMEM columns each): while one waits on its MMAs the others run epilogues
  const int grid = std::max(1, std::min(ntiles, 4 * num_sms()));
  if (v.o.fp32) {
    if (v.o.dim == 2) closure_kernel<2, true><<<grid, kTcThreads, kTcSmemBytes, st>>>(v);
    else closure_kernel<3, true><<<grid, kTcThreads, kTcSmemBytes, st>>>(v);
  } else {
    if (v.o.dim == 2) closure_kernel<2, false><<<grid, kTcThreads, kTcSmemBytes, st>>>(v);
    else closure_kernel<3, false><<<grid, kTcThreads, kTcSmemBytes, st>>>(v);
  }
}
}  // namespace psph

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct psph_mlp {
  std::string err;
  float* d_params = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  float* d_grad = nullptr;
  float* d_norm = nullptr;
  MlpImage* d_img = nullptr;
  bool img_dirty = true;
  std::vector<float> norm = std::vector<float>(PSPH_MLP_NNORM, 0.f);
  long long adam_t = 0;
  // training data
  float* d_X = nullptr;
  float* d_Y = nullptr;
  float* d_W = nullptr;  // per-sample loss weights (mean 1), or none
  int64_t n_data = 0;
  // minibatch scratch
  int cap = 0, nchunk_cap = 0;
  int* d_idx = nullptr;
  float *d_U = nullptr, *d_Z1 = nullptr, *d_Z2 = nullptr, *d_Z3 = nullptr, *d_Z4 = nullptr, *d_G4 = nullptr;
  float *d_D1 = nullptr, *d_D2 = nullptr, *d_D3 = nullptr, *d_part = nullptr;
  float* d_mma = nullptr;            // per-CTA tensor-core partials of dW3, dW2
  TrainImages* d_timg = nullptr;     // operand images of the current parameters
  int mma_cap = 0;
  double* d_loss = nullptr;
  int* d_status = nullptr;
};

namespace {

psph_status mlp_err(psph_mlp* m, psph_status code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (m) m->err = buf;
  return code;
}

#define MLP_TRY(m, call)                                                                                  \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess)                                                                                \
      return mlp_err(m, e_ == cudaErrorMemoryAllocation ? PSPH_ERR_OUT_OF_MEMORY : PSPH_ERR_CUDA, "%s: %s", #call, \
                     cudaGetErrorString(e_));                                                             \
  } while (0)

template <class T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

// CTAs of train_tc_kernel for a minibatch of B samples
int train_ctas(int B) { return std::max(1, std::min((B + kMlpTile - 1) / kMlpTile, num_sms())); }

psph_status ensure_batch(psph_mlp* m, int B) {
  const int nchunk = (B + 127) / 128;
  const int nctas = train_ctas(B);
  if (!m->d_timg) MLP_TRY(m, cudaMalloc(&m->d_timg, sizeof(TrainImages)));
  if (nctas > m->mma_cap) {
    dfree(m->d_mma);
    MLP_TRY(m, cudaMalloc(&m->d_mma, (size_t)nctas * 2 * kMlpH * kMlpH * sizeof(float)));
    m->mma_cap = nctas;
  }
  if (B <= m->cap && nchunk <= m->nchunk_cap) return PSPH_OK;
  for (float** p : {&m->d_U, &m->d_Z1, &m->d_Z2, &m->d_Z3, &m->d_Z4, &m->d_G4, &m->d_D1, &m->d_D2, &m->d_D3,
                    &m->d_part})
    dfree(*p);
  dfree(m->d_idx);
  dfree(m->d_loss);
  const size_t b = (size_t)B;
  MLP_TRY(m, cudaMalloc(&m->d_idx, b * sizeof(int)));
  MLP_TRY(m, cudaMalloc(&m->d_U, 8 * b * sizeof(float)));
  MLP_TRY(m, cudaMemset(m->d_U, 0, 8 * b * sizeof(float)));
  for (float** p : {&m->d_Z1, &m->d_Z2, &m->d_Z3, &m->d_D1, &m->d_D2, &m->d_D3})
    MLP_TRY(m, cudaMalloc(p, (size_t)kMlpH * b * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_Z4, b * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_G4, b * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_part, (size_t)nchunk * kNParams * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_loss, (size_t)((B + kTrainThreads - 1) / kTrainThreads) * sizeof(double)));
  m->cap = B;
  m->nchunk_cap = nchunk;
  return PSPH_OK;
}

// Loss and gradient of one minibatch (rows idx of X/Y, or the first B rows).
psph_status batch_grad(psph_mlp* m, const float* dX, const float* dY, const float* dW, const int* d_idx, int B,
                       double* loss) {
  psph_status st = ensure_batch(m, B);
  if (st) return st;
  const int nb = (B + kTrainThreads - 1) / kTrainThreads;
  MLP_TRY(m, ensure_train_attrs());
  // tensor cores: forward, loss gradient, deltas, dW2 / dW3
  train_images_kernel<<<(5 * kMlpH * kMlpH + 255) / 256, 256>>>(m->d_params, m->d_timg);
  MLP_TRY(m, cudaMemset(m->d_status, 0, sizeof(int)));
  const int nctas = train_ctas(B);
  train_tc_kernel<<<nctas, kTcThreads, kTrSmemBytes>>>(m->d_timg, m->d_params, m->d_norm, dX, dY, dW, d_idx, B,
                                                       m->d_U, m->d_Z1, m->d_Z2, m->d_Z3, m->d_Z4, m->d_G4, m->d_D1,
                                                       m->d_D2, m->d_D3, m->d_loss, m->d_mma, m->d_status);
  // CUDA cores: W1, the biases and the output layer, per chunk of samples
  const int chunk = 128, nchunk = (B + chunk - 1) / chunk;
  dim3 grid((kNParams + 127) / 128, nchunk);
  train_wgrad_kernel<<<grid, 128>>>(m->d_U, m->d_Z1, m->d_Z2, m->d_Z3, m->d_G4, m->d_D1, m->d_D2, m->d_D3, B, chunk,
                                    m->d_part);
  train_reduce_kernel<<<(kNParams + 127) / 128, 128>>>(m->d_part, nchunk, m->d_mma, nctas, m->d_grad);
  MLP_TRY(m, cudaGetLastError());
  int tstatus = 0;
  MLP_TRY(m, cudaMemcpy(&tstatus, m->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (tstatus) return mlp_err(m, PSPH_ERR_CUDA, "training: a tensor-core completion wait gave up");
  if (loss) {
    std::vector<double> parts(nb);
    MLP_TRY(m, cudaMemcpy(parts.data(), m->d_loss, nb * sizeof(double), cudaMemcpyDeviceToHost));
    double s = 0.0;
    for (double x : parts) s += x;
    *loss = s / B;
  }
  return PSPH_OK;
}

psph_status build_image(psph_mlp* m) {
  if (!m->img_dirty) return PSPH_OK;
  std::vector<float> p(kNParams);
  MLP_TRY(m, cudaMemcpy(p.data(), m->d_params, kNParams * sizeof(float), cudaMemcpyDeviceToHost));
  std::vector<uint8_t> buf(sizeof(MlpImage), 0);
  MlpImage* img = reinterpret_cast<MlpImage*>(buf.data());
  std::vector<float> w1(kMlpH * 16, 0.f);  // K padded to one 16-wide MMA step
  for (int r = 0; r < kMlpH; ++r)
    for (int k = 0; k < kMlpIn; ++k) w1[r * 16 + k] = p[kOW1 + r * kMlpIn + k];
  put_operand(img->w1, w1.data(), kMlpH, 16);
  put_operand(img->w2, &p[kOW2], kMlpH, kMlpH);
  put_operand(img->w3, &p[kOW3], kMlpH, kMlpH);
  std::memcpy(img->b1, &p[kOB1], kMlpH * 4);
  std::memcpy(img->b2, &p[kOB2], kMlpH * 4);
  std::memcpy(img->b3, &p[kOB3], kMlpH * 4);
  std::memcpy(img->w4, &p[kOW4], kMlpH * 4);
  img->b4 = p[kOB4];
  std::memcpy(img->mean, m->norm.data(), PSPH_MLP_NNORM * 4);
  MLP_TRY(m, cudaMemcpy(m->d_img, buf.data(), sizeof(MlpImage), cudaMemcpyHostToDevice));
  m->img_dirty = false;
  return PSPH_OK;
}

}  // namespace

psph_status psph_mlp_image(const psph_mlp* mlp, const MlpImage** dev_image) {
  psph_mlp* m = const_cast<psph_mlp*>(mlp);
  if (!m || !dev_image) return PSPH_ERR_INVALID_ARGUMENT;
  psph_status st = build_image(m);
  if (st) return st;
  *dev_image = m->d_img;
  return PSPH_OK;
}

extern "C" {

psph_status psph_mlp_create(uint64_t seed, psph_mlp** out) {
  if (!out) return PSPH_ERR_INVALID_ARGUMENT;
  psph_mlp* m = new psph_mlp();
  *out = m;
  int ndev = 0;
  if (psph_device_check(&ndev) != PSPH_OK) return mlp_err(m, PSPH_ERR_NO_DEVICE, "no sm_103 CUDA device available");
  MLP_TRY(m, cudaMalloc(&m->d_params, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_m, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_v, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_grad, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_norm, PSPH_MLP_NNORM * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_img, sizeof(MlpImage)));
  MLP_TRY(m, cudaMalloc(&m->d_status, sizeof(int)));
  MLP_TRY(m, cudaMemset(m->d_m, 0, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMemset(m->d_v, 0, kNParams * sizeof(float)));
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases; the output
  // bias starts at softplus^-1(0.02)
  std::vector<float> p(kNParams);
  uint64_t s = seed ^ 0x5eed5eedull;
  auto fill = [&](int off, int count, int fan_in) {
    const double a = 1.0 / std::sqrt((double)fan_in);
    for (int k = 0; k < count; ++k) p[off + k] = (float)((2.0 * uniform01(s) - 1.0) * a);
  };
  fill(kOW1, kMlpH * kMlpIn, kMlpIn);
  fill(kOB1, kMlpH, kMlpIn);
  fill(kOW2, kMlpH * kMlpH, kMlpH);
  fill(kOB2, kMlpH, kMlpH);
  fill(kOW3, kMlpH * kMlpH, kMlpH);
  fill(kOB3, kMlpH, kMlpH);
  fill(kOW4, kMlpH, kMlpH);
  p[kOB4] = (float)std::log(std::expm1(0.02));
  MLP_TRY(m, cudaMemcpy(m->d_params, p.data(), kNParams * sizeof(float), cudaMemcpyHostToDevice));
  for (int k = 0; k < kMlpIn; ++k) {
    m->norm[k] = 0.f;                  // mean
    m->norm[kMlpIn + k] = 1.f;         // 1/std
    m->norm[2 * kMlpIn + k] = -1e30f;  // lo
    m->norm[3 * kMlpIn + k] = 1e30f;   // hi
  }
  MLP_TRY(m, cudaMemcpy(m->d_norm, m->norm.data(), PSPH_MLP_NNORM * sizeof(float), cudaMemcpyHostToDevice));
  return PSPH_OK;
}

void psph_mlp_destroy(psph_mlp* m) {
  if (!m) return;
  cudaDeviceSynchronize();
  for (float** p : {&m->d_params, &m->d_m, &m->d_v, &m->d_grad, &m->d_norm, &m->d_X, &m->d_Y, &m->d_W, &m->d_U, &m->d_Z1,
                    &m->d_Z2, &m->d_Z3, &m->d_Z4, &m->d_G4, &m->d_D1, &m->d_D2, &m->d_D3, &m->d_part})
    dfree(*p);
  dfree(m->d_img);
  dfree(m->d_timg);
  dfree(m->d_mma);
  dfree(m->d_idx);
  dfree(m->d_loss);
  dfree(m->d_status);
  delete m;
}

const char* psph_mlp_last_error(const psph_mlp* m) { return m ? m->err.c_str() : "null network"; }

psph_status psph_mlp_set_params(psph_mlp* m, const float* params, const float* norm) {
  if (!m || (!params && !norm)) return PSPH_ERR_INVALID_ARGUMENT;
  if (params) MLP_TRY(m, cudaMemcpy(m->d_params, params, kNParams * sizeof(float), cudaMemcpyHostToDevice));
  if (norm) {
    m->norm.assign(norm, norm + PSPH_MLP_NNORM);
    MLP_TRY(m, cudaMemcpy(m->d_norm, norm, PSPH_MLP_NNORM * sizeof(float), cudaMemcpyHostToDevice));
  }
  MLP_TRY(m, cudaMemset(m->d_m, 0, kNParams * sizeof(float)));
  MLP_TRY(m, cudaMemset(m->d_v, 0, kNParams * sizeof(float)));
  m->adam_t = 0;
  m->img_dirty = true;
  return PSPH_OK;
}

psph_status psph_mlp_get_params(const psph_mlp* mlp, float* params, float* norm) {
  psph_mlp* m = const_cast<psph_mlp*>(mlp);
  if (!m) return PSPH_ERR_INVALID_ARGUMENT;
  if (params) MLP_TRY(m, cudaMemcpy(params, m->d_params, kNParams * sizeof(float), cudaMemcpyDeviceToHost));
  if (norm) std::memcpy(norm, m->norm.data(), PSPH_MLP_NNORM * sizeof(float));
  return PSPH_OK;
}

psph_status psph_mlp_set_data(psph_mlp* m, const float* x, const float* y, int64_t n) {
  if (!m || !x || !y || n < 1 || n > (1LL << 30)) return PSPH_ERR_INVALID_ARGUMENT;
  dfree(m->d_X);
  dfree(m->d_Y);
  dfree(m->d_W);
  MLP_TRY(m, cudaMalloc(&m->d_X, (size_t)n * kMlpIn * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&m->d_Y, (size_t)n * sizeof(float)));
  MLP_TRY(m, cudaMemcpy(m->d_X, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  MLP_TRY(m, cudaMemcpy(m->d_Y, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  m->n_data = n;
  for (int k = 0; k < kMlpIn; ++k) {
    double s = 0.0, s2 = 0.0, lo = x[k], hi = x[k];
    for (int64_t i = 0; i < n; ++i) {
      const double v = x[(size_t)kMlpIn * i + k];
      s += v;
      s2 += v * v;
      lo = std::min(lo, v);
      hi = std::max(hi, v);
    }
    const double mean = s / n;
    const double var = std::max(s2 / n - mean * mean, 0.0);
    const double sd = std::sqrt(var);
    const double pad = 0.05 * (hi - lo);
    m->norm[k] = (float)mean;
    m->norm[kMlpIn + k] = (float)(sd > 1e-12 ? 1.0 / sd : 1.0);
    m->norm[2 * kMlpIn + k] = (float)(lo - pad);
    m->norm[3 * kMlpIn + k] = (float)(hi + pad);
  }
  MLP_TRY(m, cudaMemcpy(m->d_norm, m->norm.data(), PSPH_MLP_NNORM * sizeof(float), cudaMemcpyHostToDevice));
  m->img_dirty = true;
  return PSPH_OK;
}

psph_status psph_mlp_set_weights(psph_mlp* m, const float* w) {
  if (!m) return PSPH_ERR_INVALID_ARGUMENT;
  if (!m->n_data) return mlp_err(m, PSPH_ERR_STATE, "psph_mlp_set_weights before psph_mlp_set_data");
  dfree(m->d_W);
  if (!w) return PSPH_OK;
  double s = 0.0;
  for (int64_t i = 0; i < m->n_data; ++i) {
    if (!(w[i] >= 0.0f) || !std::isfinite(w[i])) return mlp_err(m, PSPH_ERR_INVALID_ARGUMENT, "weight %lld is not a finite non-negative number", (long long)i);
    s += w[i];
  }
  if (!(s > 0.0)) return mlp_err(m, PSPH_ERR_INVALID_ARGUMENT, "weights sum to zero");
  std::vector<float> wn(m->n_data);
  const double scale = (double)m->n_data / s;  // mean weight 1
  for (int64_t i = 0; i < m->n_data; ++i) wn[i] = (float)(w[i] * scale);
  MLP_TRY(m, cudaMalloc(&m->d_W, (size_t)m->n_data * sizeof(float)));
  MLP_TRY(m, cudaMemcpy(m->d_W, wn.data(), (size_t)m->n_data * sizeof(float), cudaMemcpyHostToDevice));
  return PSPH_OK;
}

psph_status psph_mlp_train(psph_mlp* m, int64_t steps, int batch, float lr, uint64_t seed, float* losses) {
  if (!m || steps < 0 || batch < 1 || !(lr > 0.f)) return PSPH_ERR_INVALID_ARGUMENT;
  if (!m->n_data) return mlp_err(m, PSPH_ERR_STATE, "psph_mlp_train before psph_mlp_set_data");
  const int B = (int)std::min<int64_t>(batch, m->n_data);
  std::vector<int> perm(m->n_data);
  for (int64_t i = 0; i < m->n_data; ++i) perm[i] = (int)i;
  uint64_t rs = seed;
  int64_t pos = m->n_data;  // forces a shuffle on the first step
  psph_status st = ensure_batch(m, B);
  if (st) return st;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int64_t step = 0; step < steps; ++step) {
    if (pos + B > m->n_data) {  // new pass: Fisher-Yates with the seeded generator
      for (int64_t i = m->n_data - 1; i > 0; --i) {
        const int64_t j = (int64_t)(splitmix(rs) % (uint64_t)(i + 1));
        std::swap(perm[i], perm[j]);
      }
      pos = 0;
    }
    MLP_TRY(m, cudaMemcpy(m->d_idx, perm.data() + pos, B * sizeof(int), cudaMemcpyHostToDevice));
    pos += B;
    double loss = 0.0;
    if ((st = batch_grad(m, m->d_X, m->d_Y, m->d_W, m->d_idx, B, losses ? &loss : nullptr))) return st;
    m->adam_t += 1;
    const float c1 = (float)(1.0 - std::pow((double)b1, (double)m->adam_t));
    const float c2 = (float)(1.0 - std::pow((double)b2, (double)m->adam_t));
    adam_kernel<<<(kNParams + 255) / 256, 256>>>(m->d_params, m->d_grad, m->d_m, m->d_v, lr, b1, b2, c1, c2, eps);
    MLP_TRY(m, cudaGetLastError());
    if (losses) losses[step] = (float)loss;
  }
  MLP_TRY(m, cudaDeviceSynchronize());
  m->img_dirty = true;
  return PSPH_OK;
}

psph_status psph_mlp_loss_grad(psph_mlp* m, const float* x, const float* y, int64_t n, double* loss, float* grad) {
  if (!m || !x || !y || n < 1 || n > (1 << 24)) return PSPH_ERR_INVALID_ARGUMENT;
  float *dX = nullptr, *dY = nullptr;
  MLP_TRY(m, cudaMalloc(&dX, (size_t)n * kMlpIn * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&dY, (size_t)n * sizeof(float)));
  MLP_TRY(m, cudaMemcpy(dX, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  MLP_TRY(m, cudaMemcpy(dY, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  double l = 0.0;
  psph_status st = batch_grad(m, dX, dY, nullptr, nullptr, (int)n, &l);
  if (!st && grad) {
    cudaError_t e = cudaMemcpy(grad, m->d_grad, kNParams * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = mlp_err(m, PSPH_ERR_CUDA, "gradient copy: %s", cudaGetErrorString(e));
  }
  cudaFree(dX);
  cudaFree(dY);
  if (loss) *loss = l;
  return st;
}

psph_status psph_mlp_infer(psph_mlp* m, const float* x, int64_t n, float* c, int tensor_cores) {
  if (!m || !x || !c || n < 1 || n > (1 << 28)) return PSPH_ERR_INVALID_ARGUMENT;
  psph_status st = build_image(m);
  if (st) return st;
  float *dX = nullptr, *dC = nullptr;
  MLP_TRY(m, cudaMalloc(&dX, (size_t)n * kMlpIn * sizeof(float)));
  MLP_TRY(m, cudaMalloc(&dC, (size_t)n * sizeof(float)));
  MLP_TRY(m, cudaMemcpy(dX, x, (size_t)n * kMlpIn * sizeof(float), cudaMemcpyHostToDevice));
  MLP_TRY(m, cudaMemset(m->d_status, 0, sizeof(int)));
  if (tensor_cores) {
    MLP_TRY(m, ensure_tc_attrs());
    const int ntiles = (int)((n + kMlpTile - 1) / kMlpTile);
    const int grid = std::max(1, std::min(ntiles, 2 * num_sms()));
    infer_tc_kernel<<<grid, kTcThreads, kTcSmemBytes>>>(m->d_img, dX, (int)n, dC, m->d_status);
  } else {
    infer_cc_kernel<<<(int)((n + 127) / 128), 128>>>(m->d_params, m->d_norm, dX, (int)n, dC);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int status = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&status, m->d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(c, dC, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dX);
  cudaFree(dC);
  if (e != cudaSuccess) return mlp_err(m, PSPH_ERR_CUDA, "inference: %s", cudaGetErrorString(e));
  if (status) return mlp_err(m, PSPH_ERR_CUDA, "inference: a tensor-core completion wait gave up");
  return PSPH_OK;
}

}  // extern "C"
