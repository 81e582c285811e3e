// FP32-compensated form of the fluid pair path (precision = PSPH_FP32C).
//
// Same algorithm as psph_forces.cu (CalcForce11, Source/Interaction.cpp:25-184,
// and the wall interpolation of PrimaryComputeAcceleration,
// Source/Domain.cpp:1029-1059/:1164-1206), with the pair arithmetic in FP32:
//  - positions enter the pair kernels as (int cell, FP32 offset from the cell
//    origin); a pair's separation is (cell_i - cell_j) * CellSize + (off_i -
//    off_j), exact in the cell part and ~1e-9 m in the offset part, and the
//    periodic minimum image falls out of the wrapped cell difference;
//  - kernel, gradient, EOS-derived terms and viscosity in FP32;
//  - the acceleration and density-rate sums are Kahan-compensated in FP32;
//  - integration, material update and the dt reduction stay in FP64
//    (psph_update.cu, dt_finalize_kernel).
#include <cfloat>

#include "psph_pairs.cuh"

namespace psph {

namespace {

constexpr int kFT32 = 128;
// Minimum resident blocks per SM asked of the register allocator for the pair
// kernel (1 = no limit: ~123 registers, 4 blocks per SM).
#ifndef PSPH_FT32_MINB
#define PSPH_FT32_MINB 1
#endif
constexpr int kQ32 = 16;  // queued wall-interpolation partners per lane

struct Kahan {
  float s = 0.f, c = 0.f;
  PSPH_D void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  PSPH_D double value() const { return (double)s - (double)c; }
};

template <int DIM, int KT>
struct KernF {
  static constexpr float cw() { return (float)Kern<DIM, KT>::cw(); }
  static PSPH_D float W(float q, float cwh) {
    if (KT == 0) {
      if (q < 1.f) return cwh * (1.f - 1.5f * q * q + 0.75f * q * q * q);
      if (q < 2.f) { const float t = 2.f - q; return cwh * (0.25f * t * t * t); }
      return 0.f;
    } else if (KT == 1) {
      if (q < 2.f) { const float t = 1.f - 0.5f * q; const float t2 = t * t; return cwh * (t2 * t2) * (2.f * q + 1.f); }
      return 0.f;
    } else {
      const float a = 3.f - q, b = 2.f - q, c = 1.f - q;
      const float a2 = a * a, b2 = b * b, c2 = c * c;
      if (q < 1.f) return cwh * (a2 * a2 * a - 6.f * b2 * b2 * b + 15.f * c2 * c2 * c);
      if (q < 2.f) return cwh * (a2 * a2 * a - 6.f * b2 * b2 * b);
      if (q < 3.f) return cwh * (a2 * a2 * a);
      return 0.f;
    }
  }
  static PSPH_D float GK(float q, float inv_q, float cwg) {
    if (KT == 0) {
      if (q < 1.f) return cwg * (-3.f + 2.25f * q);
      if (q < 2.f) { const float t = 2.f - q; return cwg * inv_q * (-0.75f * t * t); }
      return 0.f;
    } else if (KT == 1) {
      if (q < 2.f) { const float t = 1.f - 0.5f * q; return cwg * -5.f * (t * t * t); }
      return 0.f;
    } else {
      const float a = 3.f - q, b = 2.f - q, c = 1.f - q;
      const float a2 = a * a, b2 = b * b, c2 = c * c;
      if (q == 0.f) return cwg * (20.f * a2 * a - 120.f * b2 * b + 300.f * c2 * c);
      if (q < 1.f) return cwg * inv_q * (-5.f * a2 * a2 + 30.f * b2 * b2 - 75.f * c2 * c2);
      if (q < 2.f) return cwg * inv_q * (-5.f * a2 * a2 + 30.f * b2 * b2);
      if (q < 3.f) return cwg * inv_q * (-5.f * a2 * a2);
      return 0.f;
    }
  }
  static PSPH_D float D2(float q, float cwg) {
    if (KT == 0) {
      if (q < 1.f) return cwg * (-3.f + 4.5f * q);
      if (q < 2.f) return cwg * (1.5f * (2.f - q));
      return 0.f;
    } else if (KT == 1) {
      if (q < 2.f) { const float t = 1.f - 0.5f * q; return cwg * (t * t) * (10.f * q - 5.f); }
      return 0.f;
    } else {
      const float a = 3.f - q, b = 2.f - q, c = 1.f - q;
      if (q < 1.f) return cwg * (20.f * a * a * a - 120.f * b * b * b + 300.f * c * c * c);
      if (q < 2.f) return cwg * (20.f * a * a * a - 120.f * b * b * b);
      if (q < 3.f) return cwg * (20.f * a * a * a);
      return 0.f;
    }
  }
  static PSPH_D float Lap(float q, float inv_q, float cwg) {
    float first;
    if (KT == 0) {
      if (q < 1.f) first = (-3.f + 2.25f * q);
      else if (q < 2.f) { const float t = 2.f - q; first = inv_q * (-0.75f * t * t); }
      else return 0.f;
    } else if (KT == 1) {
      if (q < 2.f) { const float t = 1.f - 0.5f * q; first = -5.f * t * t * t; }
      else return 0.f;
    } else {
      const float a = 3.f - q, b = 2.f - q, c = 1.f - q;
      const float a2 = a * a, b2 = b * b, c2 = c * c;
      if (q < 1.f) first = inv_q * (-5.f * a2 * a2 + 30.f * b2 * b2 - 75.f * c2 * c2);
      else if (q < 2.f) first = inv_q * (-5.f * a2 * a2 + 30.f * b2 * b2);
      else if (q < 3.f) first = inv_q * (-5.f * a2 * a2);
      else return 0.f;
    }
    return D2(q, cwg) + cwg * (DIM - 1.f) * first;
  }
};

// ---------------------------------------------------------------------------
// Preparation (FP32 copies, partner-visible wall state) and wall interpolation
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void __launch_bounds__(kFT32) copies32_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= sc->n) return;
  const PClass32& C = v.cls32[P.cls[w]];
  if (v.inst[C.inst].stop) return;
  const double4_32a vv = P.V4[w];
  const float p = (float)vv.w;
  v.S.V32[w] = make_float4((float)vv.x, (float)vv.y, (float)vv.z, p);
  if (C.flags & CF_FREE) {
    const float rho = (float)P.X4[w].w;
    const float inv = 1.f / rho;
    const float ratio = rho / C.rho0;
    const float c = (C.pres_eq == 1) ? C.cs * ratio * ratio * ratio : C.cs;
    v.S.D32[w] = make_float4(inv, p * inv * inv, c, rho);
  }
}

template <int DIM, int KT>
__global__ void __launch_bounds__(kFT32) prepare32_kernel(DevView v) {
  __shared__ int qbuf[kQ32][kFT32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const int tid = threadIdx.x;
  const Options& o = v.o;
  const PClass32* __restrict__ CT = v.cls32;
  const int winst = (w < n) ? CT[P.cls[w]].inst : 0;
  const GridDev& g = grid_of(v, winst);
  bool wall = false, noslip = false;
  int cell = -1, ow = 0, mat = 0;
  float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
  if (w < n && !v.inst[winst].stop) {
    const PClass32& C = CT[P.cls[w]];
    if (!(C.flags & CF_FREE)) {
      wall = true;
      noslip = C.flags & CF_NOSLIP;
      mat = C.material;
      ow = P.orig[w];
      cell = v.S.cellid[w];
      oi = v.S.OFF32[w];
    }
  }
  const float3 cs = cell_size_f(g);
  const float gx = (float)o.gravity[0], gy = (float)o.gravity[1], gz = (float)o.gravity[2];
  const bool need_orient = !o.wallp_physical && (gx != 0.f || gy != 0.f || gz != 0.f);
  float sk = 0.f, p = 0.f, n0 = 0.f, n1 = 0.f, n2 = 0.f;
  NbrSource<DIM> src;
  src.init(v, g, w, wall && cell >= 0, 1.0f);
  bool more = wall && cell >= 0;
  const float hw = oi.w;
  while (true) {
    int qn = 0;
    while (more && qn < kQ32) {
      int code;
      const int f = src.next(v, &code);
      if (f < 0) {
        more = false;
        break;
      }
      qbuf[qn++][tid] = f | (code << kCodeShift);
    }
    const int qmax = __reduce_max_sync(0xffffffffu, qn);
    for (int k = 0; k < qmax; ++k) {
      if (k >= qn) continue;
      const int e = qbuf[k][tid];
      const int f = e & kIndexMask, code = e >> kCodeShift;
      const PClass32& Cf = CT[P.cls[f]];
      if (!(Cf.flags & CF_FREE) || Cf.material != mat) continue;
      const float4 of = v.S.OFF32[f];
      float x0, x1, x2;
      rel_pos<DIM>(cs, oi, of, code, x0, x1, x2);  // x_wall - x_fluid
      if (need_orient && !first_of_pair_code(code, ow, P.orig[f])) {
        x0 = -x0; x1 = -x1; x2 = -x2;
      }
      const float hb = 0.5f * (hw + of.w);
      const float ih = 1.f / hb;
      const float q = sqrtf(x0 * x0 + x1 * x1 + x2 * x2) * ih;
      const float K = KernF<DIM, KT>::W(q, KernF<DIM, KT>::cw() * (DIM == 2 ? ih * ih : ih * ih * ih));
      if (K == 0.f) continue;
      const float4 vf = v.S.V32[f];
      const float4 df = v.S.D32[f];
      sk += K;
      p += vf.w * K + (gx * x0 + gy * x1 + gz * x2) * df.w * K;
      if (noslip) { n0 += vf.x * K; n1 += vf.y * K; n2 += vf.z * K; }
    }
    if (!__any_sync(0xffffffffu, more)) break;
  }
  if (!wall) return;
  if (sk != 0.f) {
    p = p / sk;
    if (noslip) { n0 /= sk; n1 /= sk; n2 /= sk; }
  } else {
    p = 0.f; n0 = n1 = n2 = 0.f;
  }
  double4_32a vw = P.V4[w];
  vw.w = (double)p;
  P.V4[w] = vw;
  v.S.sumkernel[w] = sk;
  v.S.nsv4[w] = make_double4_32a(n0, n1, n2, 0.0);
  v.S.V32[w] = make_float4((float)vw.x, (float)vw.y, (float)vw.z, p);
  const PClass32& Ce = CT[o.eos_cls];
  float rw = (float)P.X4[w].w, cwv = 0.f;
  if (o.uniform_eos) {
    // DensitySolid / SoundSpeed of the fluid's EOS (Source/Functions.cpp:214-264), FP32
    const float cs2 = Ce.cs * Ce.cs, r0 = Ce.rho0, p0 = Ce.p0;
    if (Ce.pres_eq == 0) rw = (p - p0) / cs2 + r0;
    else if (Ce.pres_eq == 1) rw = powf((p - p0) * (7.f / (r0 * cs2)) + 1.f, 1.f / 7.f) * r0;
    else rw = p / cs2;
    const float ratio = rw / r0;
    cwv = (Ce.pres_eq == 1) ? Ce.cs * ratio * ratio * ratio : Ce.cs;
  }
  const float inv = 1.f / rw;
  v.S.D32[w] = make_float4(inv, p * inv * inv, cwv, rw);
}

// ---------------------------------------------------------------------------
// Fluid pair force, FP32 with compensated sums, over the neighbour lists
// ---------------------------------------------------------------------------
template <int DIM, int KT>
__global__ void __launch_bounds__(kFT32, PSPH_FT32_MINB) forces_fluid32_kernel(DevView v) {
  __shared__ double red[kFT32 / 32];
  __shared__ unsigned long long cred[kFT32 / 32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int tid = threadIdx.x;
  const Options& o = v.o;
  const PClass32* __restrict__ CT = v.cls32;
  double dtc = DBL_MAX;
  unsigned long long npair2 = 0;
  bool active = false;
  int cell = -1, ci_cls = 0;
  if (i < n) {
    ci_cls = P.cls[i];
    const bool run = !v.inst[CT[ci_cls].inst].stop;
    active = run && (CT[ci_cls].flags & CF_FREE);
    cell = v.S.cellid[i];
    if (run && !active) {
      v.S.A4[i] = make_double4_32a(o.gravity[0], o.gravity[1], o.gravity[2], 0.0);
      v.S.zwab[i] = 1.0;
    }
  }
  const PClass32& Ci = CT[ci_cls];
  const GridDev& g = grid_of(v, Ci.inst);
  const InstState& Is = v.inst[Ci.inst];
  const int is = active ? i : 0;
  const float4 oi = v.S.OFF32[is];
  const float4 vi = v.S.V32[is];
  const float4 di4 = v.S.D32[is];
  const float di = di4.w, inv_i = di4.x, Pi = di4.y, ci_snd = di4.z, pi = vi.w;
  const float mi = Ci.mass, hi = oi.w;
  const float mui = o.dyn_mu ? (float)P.mu[is] : Ci.mu0;
  const int fi = Ci.flags;
  const bool shep = (fi & CF_SHEPARD) && (Is.shepard_counter == o.shepard_step);
  const bool sr_self = fi & (CF_T0 | CF_LES);
  const bool use_sr = o.need_sr;
  const bool xsph_on = o.xsph != 0.0;
  const float xsph = (float)o.xsph;
  const float3 cs = cell_size_f(g);
  const float mu_u = (float)o.mu_u;
  const bool uniform_mu = o.uniform_mu, dyn_mu = o.dyn_mu;
  const int vis_eq = o.vis_eq, grad_type = o.grad_type;
  Kahan ax, ay, az, dr;
  float zw = 0.f, sd = 0.f, xs0 = 0.f, xs1 = 0.f, xs2 = 0.f;
  float sr0 = 0.f, sr1 = 0.f, sr2 = 0.f, sr4 = 0.f, sr5 = 0.f, sr8 = 0.f;
  float w01 = 0.f, w02 = 0.f, w12 = 0.f;  // antisymmetric counterpart of the strain-rate sums (closure)
  int nnb = 0;
  const bool closure = o.closure && (fi & CF_LES);
  NbrSource<DIM> src;
  src.init(v, g, i, active && cell >= 0, 1.0f);
  while (true) {
    int code;
    const int j = src.next(v, &code);
    if (j < 0) break;
    const float4 oj = v.S.OFF32[j];
    float x0, x1, x2;
    rel_pos<DIM>(cs, oi, oj, code, x0, x1, x2);
    const PClass32& Cj = CT[P.cls[j]];
    const int fjf = Cj.flags;
    const bool fj = fjf & CF_FREE;
    npair2 += fj ? 1ull : 2ull;
    ++nnb;
    const float hb = 0.5f * (hi + oj.w);
    const float ih = 1.f / hb;
    const float r2 = x0 * x0 + x1 * x1 + x2 * x2;
    const float inv_r = (r2 > 0.f) ? rsqrtf(r2) : 0.f;
    const float q = r2 * inv_r * ih;
    const float inv_q = hb * inv_r;
    const float ih2 = ih * ih;
    const float cwh = KernF<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * ih);
    const float cwg = cwh * ih2;
    const float GK = KernF<DIM, KT>::GK(q, inv_q, cwg);
    const float K = KernF<DIM, KT>::W(q, cwh);
    const float4 vj = v.S.V32[j];
    const float4 dj4 = v.S.D32[j];
    const float dj = dj4.w, inv_j = dj4.x, Pj = dj4.y, cj_snd = dj4.z, pj = vj.w;
    const float mj = fj ? Cj.mass : Cj.fpmassc * mi;
    const float v0 = vi.x - vj.x, v1 = vi.y - vj.y, v2 = vi.z - vj.z;
    const float vx = v0 * x0 + v1 * x1 + v2 * x2;
    float PI = 0.f;
    const float Alpha = 0.5f * (Ci.alpha + Cj.alpha), Beta = 0.5f * (Ci.beta + Cj.beta);
    if ((Alpha != 0.f || Beta != 0.f) && vx < 0.f) {
      const float D = r2 + 0.01f * hb * hb;
      const float t = hb * vx;
      PI = t * (-Alpha * 0.5f * (ci_snd + cj_snd) * D + Beta * t) / (D * D * (0.5f * (di + dj)));
    }
    float TI = 0.f;
    if ((fi | fjf) & CF_TI) {
      float Ri = 0.f, Rj = 0.f;
      if ((pi + pj) < 0.f) {
        if (pi < 0.f) Ri = -pi * inv_i * inv_i;
        if (pj < 0.f) Rj = -pj * inv_j * inv_j;
      }
      const float Wd = KernF<DIM, KT>::W((Ci.tid + Cj.tid) * 0.5f * ih, cwh);
      TI = (Ci.ti * Ri + Cj.ti * Rj) * powf(K / Wd, (Ci.tin + Cj.tin) * 0.5f);
    }
    float VI0 = 0.f, VI1 = 0.f, VI2 = 0.f;
    if (((fi | fjf) & CF_NOSLIP) || fj) {
      float Mu, vab0, vab1, vab2;
      if (fj) {
        vab0 = v0; vab1 = v1; vab2 = v2;
        if (uniform_mu) Mu = mu_u;
        else {
          const float muj = dyn_mu ? (float)P.mu[j] : Cj.mu0;
          Mu = 2.f * mui * muj / (mui + muj);
        }
      } else {
        const double4_32a ns = v.S.nsv4[j];
        vab0 = vi.x - (2.f * vj.x - (float)ns.x);
        vab1 = vi.y - (2.f * vj.y - (float)ns.y);
        vab2 = vi.z - (2.f * vj.z - (float)ns.z);
        Mu = mui;
      }
      if (vis_eq <= 2) {
        float c;
        if (vis_eq == 0) c = 2.f * Mu * inv_i * inv_j * GK;
        else if (vis_eq == 1) c = 8.f * Mu / ((di + dj) * (di + dj)) * GK;
        else c = -Mu * inv_i * inv_j * KernF<DIM, KT>::Lap(q, inv_q, cwg);
        VI0 = c * vab0; VI1 = c * vab1; VI2 = c * vab2;
      } else {
        const float L = KernF<DIM, KT>::Lap(q, inv_q, cwg);
        const float S2 = KernF<DIM, KT>::D2(q, cwg);
        const float s = -Mu * inv_i * inv_j;
        const float t = vx / r2 * (-GK + S2);
        VI0 = s * (L * vab0 + (1.f / 3.f) * (GK * v0 + t * x0));
        VI1 = s * (L * vab1 + (1.f / 3.f) * (GK * v1 + t * x1));
        VI2 = s * (L * vab2 + (1.f / 3.f) * (GK * v2 + t * x2));
      }
      if (use_sr && sr_self && (((fi | fjf) & CF_T0) || ((fi & fjf) & CF_LES))) {
        const float c2 = -GK * (mj * inv_j);
        sr0 += c2 * (2.f * vab0 * x0);
        sr1 += c2 * (vab0 * x1 + vab1 * x0);
        sr2 += c2 * (vab0 * x2 + vab2 * x0);
        sr4 += c2 * (2.f * vab1 * x1);
        sr5 += c2 * (vab1 * x2 + vab2 * x1);
        sr8 += c2 * (2.f * vab2 * x2);
        if (closure) {
          w01 += c2 * (vab0 * x1 - vab1 * x0);
          w02 += c2 * (vab0 * x2 - vab2 * x0);
          w12 += c2 * (vab1 * x2 - vab2 * x1);
        }
      }
    }
    if (xsph_on && fj) {
      const float s = xsph * mj / (0.5f * (di + dj)) * K;
      xs0 -= s * v0; xs1 -= s * v1; xs2 -= s * v2;
    }
    float s;
    if (grad_type == 0) s = -(Pi + Pj + PI + TI) * GK;
    else s = -((pi + pj) * inv_i * inv_j + PI + TI) * GK;
    ax.add(mj * (s * x0 + VI0));
    ay.add(mj * (s * x1 + VI1));
    if (DIM == 3) az.add(mj * (s * x2 + VI2));
    dr.add(mj * di * inv_j * (GK * vx));
    zw += mj * inv_j * K;
    if (shep) sd += mj * K;
  }
  if (active) {
    const double axd = o.gravity[0] + o.body_force[0] + ax.value();
    const double ayd = o.gravity[1] + o.body_force[1] + ay.value();
    const double azd = o.gravity[2] + o.body_force[2] + az.value();
    const double drd = dr.value();
    v.S.A4[i] = make_double4_32a(axd, ayd, azd, drd);
    v.S.zwab[i] = zw;
    if (o.any_shepard) v.S.sumden[i] = sd;
    if (xsph_on) v.S.vxsph4[i] = make_double4_32a(xs0, xs1, xs2, 0.0);
    if (use_sr) {
      double* out = v.S.strain_rate + 9 * (size_t)i;
      out[0] = sr0; out[1] = sr1; out[2] = sr2;
      out[3] = sr1; out[4] = sr4; out[5] = sr5;
      out[6] = sr2; out[7] = sr5; out[8] = sr8;
    }
    if (closure) {
      v.S.cvort[i] = sqrtf(w01 * w01 + w02 * w02 + w12 * w12);
      v.S.cnnb[i] = (float)nnb;
    }
    if (!(isfinite(axd) && isfinite(ayd) && isfinite(azd) && isfinite(drd))) atomicOr(&v.sc->status, ST_NONFINITE);
    const double an = sqrt(axd * axd + ayd * ayd + azd * azd);
    const double cand = o.sqrt_h_a * sqrt(v.cls[ci_cls].h / an);  // FP64 dt reduction
    if (cand < dtc) dtc = cand;
  }
  block_dt_and_pairs<kFT32>(v, Ci.inst, active, dtc, npair2, red, cred);
}

inline int nblk32(int n) { return n <= 0 ? 1 : (n + kFT32 - 1) / kFT32; }

template <int DIM>
void prepare32_dispatch(const DevView& v, cudaStream_t st) {
  const int nb = nblk32(v.ncap);
  copies32_kernel<DIM><<<nb, kFT32, 0, st>>>(v);
  switch (v.o.kt) {
    case 0: prepare32_kernel<DIM, 0><<<nb, kFT32, 0, st>>>(v); break;
    case 1: prepare32_kernel<DIM, 1><<<nb, kFT32, 0, st>>>(v); break;
    default: prepare32_kernel<DIM, 2><<<nb, kFT32, 0, st>>>(v); break;
  }
}

template <int DIM>
void forces32_dispatch(const DevView& v, cudaStream_t st) {
  const int nb = nblk32(v.ncap);
  switch (v.o.kt) {
    case 0: forces_fluid32_kernel<DIM, 0><<<nb, kFT32, 0, st>>>(v); break;
    case 1: forces_fluid32_kernel<DIM, 1><<<nb, kFT32, 0, st>>>(v); break;
    default: forces_fluid32_kernel<DIM, 2><<<nb, kFT32, 0, st>>>(v); break;
  }
}

}  // namespace

void launch_prepare32(const DevView& v, cudaStream_t st) {
  if (v.o.dim == 2) prepare32_dispatch<2>(v, st);
  else prepare32_dispatch<3>(v, st);
}

void launch_forces32(const DevView& v, cudaStream_t st) {
  if (v.o.dim == 2) forces32_dispatch<2>(v, st);
  else forces32_dispatch<3>(v, st);
}

}  // namespace psph
