// FP32-compensated form of the pair path (precision = PSPH_FP32C): fluids
// (CalcForce11) and soil / solids (CalcForce2233).
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

constexpr int kFT32 = 128;  // block size of the copy and wall-interpolation kernels
// The pair kernels take their block size at launch (Options::pair_block, 64 to
// 256 threads, picked by psph_autotune); register caps are set per kernel.
constexpr int kMaxPairBlock = 256;

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

// Loads issued where they stand: the neighbour's velocity, density and class
// go out together with its position, ahead of the support test, so the pair
// waits for one memory round trip instead of two (a plain load would be sunk
// below the test's branch). Read-only for the kernel's lifetime.
PSPH_D float4 ld_early(const float4* p) {
  float4 r;
  asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}
PSPH_D int ld_early(const int* p) {
  int r;
  asm volatile("ld.global.nc.b32 %0, [%1];" : "=r"(r) : "l"(p));
  return r;
}
// the same for an array the kernel itself writes elsewhere (coherent path)
PSPH_D float4 ld_early_coherent(const float4* p) {
  float4 r;
  asm volatile("ld.global.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}

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
  // every conversion on the integer pipe (d2f_rn / d2f_split: the values of
  // the conversion instruction, which runs on the FP64 pipe)
  const float p = d2f_rn(vv.w);
  float lx, ly, lz;
  const float vx = d2f_split(vv.x, &lx), vy = d2f_split(vv.y, &ly), vz = d2f_split(vv.z, &lz);
  v.S.V32[w] = make_float4(vx, vy, vz, p);
  // the velocity's low-order part: in a smooth flow v_i - v_j is far smaller
  // than v, and the pair differences take (hi_i - hi_j) + (lo_i - lo_j), exact
  // to ~2^-48 of |v|; the class index and its flags ride along in .w (class |
  // flags << 16: one load per pair, and no class-table load when the pair
  // constants are uniform)
  v.S.V32LO[w] = make_float4(lx, ly, lz, __int_as_float(P.cls[w] | (C.flags << 16)));
  if (C.flags & CF_FREE) {
    const float rho = d2f_rn(P.X4[w].w);
    const float inv = 1.f / rho;
    const float ratio = rho / C.rho0;
    const float c = (C.pres_eq == 1) ? C.cs * ratio * ratio * ratio : C.cs;
    v.S.D32[w] = make_float4(inv, p * inv * inv, c, rho);
  }
  // FP32 copy of a per-particle viscosity: the pair loop then converts nothing
  // (a double-to-float conversion runs on the FP64 pipe, 1/64 of the FP32 rate)
  if (v.o.dyn_mu) v.S.MU32[w] = d2f_rn(P.mu[w]);
}

template <int DIM, int KT>
__global__ void __launch_bounds__(kFT32) prepare32_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
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
  const float gx = o.gravity32[0], gy = o.gravity32[1], gz = o.gravity32[2];
  const bool need_orient = !o.wallp_physical && (gx != 0.f || gy != 0.f || gz != 0.f);
  const bool skin = o.skin > 0.f;
  const int rc_w = (skin && need_orient && wall) ? v.S.refcell[w] : 0;
  float sk = 0.f, p = 0.f, n0 = 0.f, n1 = 0.f, n2 = 0.f;
  const float hw = oi.w;
  // one fluid neighbour of the same material: its position, velocity and
  // density loads go out together (this kernel writes the walls' own V32 /
  // D32, which the class test then rejects, so those two take the coherent path)
  auto visit = [&](const int f, const int code) {
    const int clsf = ld_early(P.cls + f);
    const float4 of = v.S.OFF32[f];
    const float4 vf = ld_early_coherent(v.S.V32 + f);
    const float4 df = ld_early_coherent(v.S.D32 + f);
    const PClass32& Cf = CT[clsf];
    if (!(Cf.flags & CF_FREE) || Cf.material != mat) return;
    float x0, x1, x2;
    rel_pos<DIM>(cs, oi, of, code, x0, x1, x2);  // x_wall - x_fluid
    if (need_orient) {
      // the pair's cell offset in the reference's grid (with a skin the lists'
      // cells are coarser): it decides which particle the reference lists first
      const int cd = skin ? ref_code(rc_w, v.S.refcell[f]) : code;
      if (!first_of_pair_code(cd, ow, P.orig[f])) {
        x0 = -x0; x1 = -x1; x2 = -x2;
      }
    }
    const float hb = 0.5f * (hw + of.w);
    const float ih = 1.f / hb;
    const float q = sqrtf(x0 * x0 + x1 * x1 + x2 * x2) * ih;
    const float K = KernF<DIM, KT>::W(q, KernF<DIM, KT>::cw() * (DIM == 2 ? ih * ih : ih * ih * ih));
    if (K == 0.f) return;
    sk += K;
    p += vf.w * K + (gx * x0 + gy * x1 + gz * x2) * df.w * K;
    if (noslip) { n0 += vf.x * K; n1 += vf.y * K; n2 += vf.z * K; }
  };
  const int cnt = (wall && cell >= 0) ? v.S.nl_count[w] : 0;
  if (cnt >= 0) {  // the neighbour list, 4 entries per 16-byte load
    const int4* __restrict__ nl4 = reinterpret_cast<const int4*>(v.S.nl) + nl_slot(w);
    const size_t N = (size_t)v.nl_stride;
    const int nch = (cnt + 3) >> 2;
    for (int c = 0; c < nch; ++c) {
      const int4 q = nl4[(size_t)c * N];
      const int rem = cnt - 4 * c;
      visit(q.x & kIndexMask, q.x >> kCodeShift);
      if (rem > 1) visit(q.y & kIndexMask, q.y >> kCodeShift);
      if (rem > 2) visit(q.z & kIndexMask, q.z >> kCodeShift);
      if (rem > 3) visit(q.w & kIndexMask, q.w >> kCodeShift);
    }
  } else {  // list overflow: scan the cells
    NbrSource<DIM> src;
    src.init(v, g, w, true, 1.0f);
    while (true) {
      int code;
      const int f = src.next(v, &code);
      if (f < 0) break;
      visit(f, code);
    }
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
  v.S.NSV32[w] = make_float4(n0, n1, n2, 0.f);
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
// FL selects a compile-time specialisation: 0 = every option read at run time;
// 1, 2 and 3 = Morris viscosity, squared-density gradient, no tensile-instability
// term, no XSPH, one h, and pair constants (artificial viscosity, masses) the
// same for every class, taken from the launch parameters instead of the class
// table (the dam-break configuration): without (1) or with (2) the strain-rate
// sums of the LES / Bingham options, or with them and the learned closure's
// vorticity (3). The list walk is a counted
// loop so that the next neighbour's loads can be issued before this one's
// arithmetic; each pair issues all of its neighbour loads before the support
// test (ld_early).
// Register caps measured on the 6.7M-particle dam break (64 to 112 swept): the
// strain-rate flavours run best at 96 (20 warps/SM), the plain one at 80, the
// general one at 128.
template <int DIM, int KT, int FL>
__global__ void __maxnreg__(FL == 0 ? 128 : (FL == 1 ? 80 : 96)) forces_fluid32_kernel(DevView v) {
  constexpr bool SPEC = FL != 0;
  constexpr bool CLOSURE = FL == 3;
  __shared__ unsigned long long cred[32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Options& o = v.o;
  const PClass32* __restrict__ CT = v.cls32;
  float dtc = FLT_MAX;
  unsigned npair2 = 0;  // 2 per pair with a free partner, 1 per wall partner (the pair is counted once)
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
  const float4 vil = v.S.V32LO[is];
  const float4 di4 = v.S.D32[is];
  const float di = di4.w, inv_i = di4.x, Pi = di4.y, ci_snd = di4.z, pi = vi.w;
  const float mi = Ci.mass, hi = oi.w;
  const float mui = o.dyn_mu ? v.S.MU32[is] : Ci.mu0;
  const int fi = Ci.flags;
  const bool shep = (fi & CF_SHEPARD) && (Is.shepard_counter == o.shepard_step);
  const bool sr_self = fi & (CF_T0 | CF_LES);
  const bool use_sr = SPEC ? (FL >= 2) : (bool)o.need_sr;
  const bool xsph_on = SPEC ? false : o.xsph != 0.0;
  const float xsph = o.xsph32;
  const float3 cs = cell_size_f(g);
  const float mu_u = o.mu_u32;
  const bool uniform_mu = o.uniform_mu, dyn_mu = o.dyn_mu;
  const int vis_eq = SPEC ? 0 : o.vis_eq, grad_type = SPEC ? 0 : o.grad_type;
  Kahan ax, ay, az, dr;
  float zw = 0.f, sd = 0.f, xs0 = 0.f, xs1 = 0.f, xs2 = 0.f;
  // strain-rate sums as sums of products a_r x_c (a = c2 vab): diagonal
  // m00 m11 m22, and the off-diagonal pairs either summed (s01 = m01 + m10 ...)
  // or, with the closure (whose vorticity needs the antisymmetric part), kept
  // apart (m01, m10, ...)
  float m00 = 0.f, m11 = 0.f, m22 = 0.f, m01 = 0.f, m02 = 0.f, m12 = 0.f, m10 = 0.f, m20 = 0.f, m21 = 0.f;
  int nnb = 0;
  const bool closure = SPEC ? (CLOSURE && (fi & CF_LES)) : (o.closure && (fi & CF_LES));
  // the closure flavour always keeps the antisymmetric sums apart
  const bool split_sr = SPEC ? CLOSURE : closure;
  const float cf2 = g.cellfac2_32;
  const bool uniform_h = o.uniform_h;
  const float ih_u = o.inv_h32;
  auto pair = [&](const int j, const int code) {
    const float4 oj = v.S.OFF32[j];
    const float4 vjl = ld_early(v.S.V32LO + j);
    const float4 vj = ld_early(v.S.V32 + j);
    const float4 dj4 = ld_early(v.S.D32 + j);
    const int wj = __float_as_int(vjl.w);
    const int clsj = wj & 0xffff;
    float x0, x1, x2;
    rel_pos<DIM>(cs, oi, oj, code, x0, x1, x2);
    const float hb = SPEC ? hi : 0.5f * (hi + oj.w);  // one h: (h + h) / 2 = h exactly
    const float r2 = x0 * x0 + x1 * x1 + x2 * x2;
    // the list's own support test (exact in FP32; lists with a skin hold more)
    if (r2 > cf2 * hb * hb) return;
    const PClass32& Cj = CT[SPEC ? 0 : clsj];
    const int fjf = wj >> 16;
    const bool fj = fjf & CF_FREE;
    npair2 += fj ? 1u : 2u;
    ++nnb;
    // FP32C divisions use the hardware reciprocal (2 ulp; the form's bound is 1e-5)
    const float ih = uniform_h ? ih_u : __fdividef(1.f, hb);
    const float inv_r = (r2 > 0.f) ? rsqrtf(r2) : 0.f;
    const float q = r2 * inv_r * ih;
    const float inv_q = hb * inv_r;
    const float ih2 = ih * ih;
    const float cwh = KernF<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * ih);
    const float cwg = cwh * ih2;
    const float GK = KernF<DIM, KT>::GK(q, inv_q, cwg);
    const float K = KernF<DIM, KT>::W(q, cwh);
    const float dj = dj4.w, inv_j = dj4.x, Pj = dj4.y, cj_snd = dj4.z, pj = vj.w;
    const float mj = SPEC ? (fj ? o.m_free32 : o.fpm_wall32 * mi) : (fj ? Cj.mass : Cj.fpmassc * mi);
    const float v0 = (vi.x - vj.x) + (vil.x - vjl.x), v1 = (vi.y - vj.y) + (vil.y - vjl.y),
                v2 = (vi.z - vj.z) + (vil.z - vjl.z);
    const float vx = v0 * x0 + v1 * x1 + v2 * x2;
    float PI = 0.f;
    const float Alpha = SPEC ? o.alpha32 : 0.5f * (Ci.alpha + Cj.alpha);
    const float Beta = SPEC ? o.beta32 : 0.5f * (Ci.beta + Cj.beta);
    if ((Alpha != 0.f || Beta != 0.f) && vx < 0.f) {
      const float D = r2 + 0.01f * hb * hb;
      const float t = hb * vx;
      PI = __fdividef(t * (-Alpha * 0.5f * (ci_snd + cj_snd) * D + Beta * t), D * D * (0.5f * (di + dj)));
    }
    float TI = 0.f;
    if (!SPEC && ((fi | fjf) & CF_TI)) {
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
          const float muj = dyn_mu ? v.S.MU32[j] : (SPEC ? Ci.mu0 : Cj.mu0);
          Mu = __fdividef(2.f * mui * muj, mui + muj);
        }
      } else {
        const float4 ns = v.S.NSV32[j];
        vab0 = (vi.x - (2.f * vj.x - ns.x)) + (vil.x - 2.f * vjl.x);
        vab1 = (vi.y - (2.f * vj.y - ns.y)) + (vil.y - 2.f * vjl.y);
        vab2 = (vi.z - (2.f * vj.z - ns.z)) + (vil.z - 2.f * vjl.z);
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
        // StrainRate += (m_j / rho_j) S with S = -GK [2 v_a x_a, v_a x_b + v_b x_a, ...]
        // (Source/Interaction.cpp:114-117, no 1/2): a = c2 vab, S_rc = a_r x_c + a_c x_r
        const float c2 = -GK * (mj * inv_j);
        const float a0 = c2 * vab0, a1 = c2 * vab1, a2 = c2 * vab2;
        m00 = fmaf(a0, x0, m00);
        m11 = fmaf(a1, x1, m11);
        m22 = fmaf(a2, x2, m22);
        m01 = fmaf(a0, x1, m01);
        m02 = fmaf(a0, x2, m02);
        m12 = fmaf(a1, x2, m12);
        if (split_sr) {
          m10 = fmaf(a1, x0, m10);
          m20 = fmaf(a2, x0, m20);
          m21 = fmaf(a2, x1, m21);
        } else {
          m01 = fmaf(a1, x0, m01);
          m02 = fmaf(a2, x0, m02);
          m12 = fmaf(a2, x1, m12);
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
  };
  const int cnt = (active && cell >= 0) ? v.S.nl_count[i] : 0;
  if (cnt >= 0) {
    const int4* __restrict__ nl4 = reinterpret_cast<const int4*>(v.S.nl) + nl_slot(i);
    const size_t N = (size_t)v.nl_stride;
    const int nch = (cnt + 3) >> 2;
    // the strain-rate flavour loads the next chunk one chunk ahead (measured:
    // it helps there and costs the plain flavour a little)
    constexpr bool kAhead = FL >= 2;
    int4 qn = (kAhead && nch > 0) ? nl4[0] : make_int4(0, 0, 0, 0);
    for (int c = 0; c < nch; ++c) {  // one 16-byte chunk of 4 entries per load
      int4 q;
      if (kAhead) {
        q = qn;
        if (c + 1 < nch) qn = nl4[(size_t)(c + 1) * N];
      } else {
        q = nl4[(size_t)c * N];
      }
      const int rem = cnt - 4 * c;
      pair(q.x & kIndexMask, q.x >> kCodeShift);
      if (rem > 1) pair(q.y & kIndexMask, q.y >> kCodeShift);
      if (rem > 2) pair(q.z & kIndexMask, q.z >> kCodeShift);
      if (rem > 3) pair(q.w & kIndexMask, q.w >> kCodeShift);
    }
  } else {  // list overflow: scan the cells
    NbrSource<DIM> src;
    src.init(v, g, i, true, 1.0f);
    while (true) {
      int code;
      const int j = src.next(v, &code);
      if (j < 0) break;
      pair(j, code);
    }
  }
  if (active) {
    const double axd = o.gb[0] + ax.value();
    const double ayd = o.gb[1] + ay.value();
    const double azd = o.gb[2] + az.value();
    const double drd = dr.value();
    v.S.A4[i] = make_double4_32a(axd, ayd, azd, drd);
    v.S.zwab[i] = zw;
    if (o.any_shepard) v.S.sumden[i] = sd;
    if (xsph_on) v.S.vxsph4[i] = make_double4_32a(xs0, xs1, xs2, 0.0);
    if (use_sr) {
      // symmetric sums 2 m_rr and m_rc + m_cr; the antisymmetric m_rc - m_cr
      // (closure) is the vorticity's
      const float sr0 = 2.f * m00, sr4 = 2.f * m11, sr8 = 2.f * m22;
      const float sr1 = split_sr ? m01 + m10 : m01, sr2 = split_sr ? m02 + m20 : m02,
                  sr5 = split_sr ? m12 + m21 : m12;
      const float w01 = m01 - m10, w02 = m02 - m20, w12 = m12 - m21;
      // the 6 distinct sums in FP32 (the FP64 tensor is built on download)
      float2* out = reinterpret_cast<float2*>(v.S.sr32 + 6 * (size_t)i);
      out[0] = make_float2(sr0, sr1);
      out[1] = make_float2(sr2, sr4);
      out[2] = make_float2(sr5, sr8);
      // Mat1's ShearRate contraction (Source/Particle.cpp:151-153) of the
      // symmetric sums, in FP32: the update and the closure take it from here
      const float temp = sr0 * sr0 + 2.f * sr1 * sr1 + 2.f * sr2 * sr2 + sr4 * sr4 + 2.f * sr5 * sr5 + sr8 * sr8;
      v.S.cshear[i] = sqrtf(0.5f * temp);
      if (closure) {
        v.S.cvort[i] = sqrtf(w01 * w01 + w02 * w02 + w12 * w12);
        v.S.cnnb[i] = (float)nnb;
        const float det =
            sr0 * (sr4 * sr8 - sr5 * sr5) - sr1 * (sr1 * sr8 - sr5 * sr2) + sr2 * (sr1 * sr5 - sr4 * sr2);
        v.S.cr3[i] = temp > 0.f ? det / (temp * sqrtf(temp)) : 0.f;
      }
    }
    // the FP64 sums are finite exactly when their FP32 parts are (checked in FP32)
    const float fin = (ax.s - ax.s) + (ax.c - ax.c) + (ay.s - ay.s) + (ay.c - ay.c) + (az.s - az.s) +
                      (az.c - az.c) + (dr.s - dr.s) + (dr.c - dr.c);
    if (!(fin == 0.f)) atomicOr(&v.sc->status, ST_NONFINITE);
    // this particle's time-step bound sqrt_h_a sqrt(h/|a|) in FP32; the
    // minimum over particles (FP32 within a warp) and AdaptiveTimeStep stay FP64
    const float ax32 = (float)axd, ay32 = (float)ayd, az32 = (float)azd;
    const float an = sqrtf(ax32 * ax32 + ay32 * ay32 + az32 * az32);
    const float cand = o.sqrt_h_a32 * sqrtf(Ci.h / an);
    if (cand < dtc) dtc = cand;
  }
  block_dt32_and_pairs(v, Ci.inst, active, dtc, (unsigned long long)npair2, cred);
}

// ---------------------------------------------------------------------------
// Soil / solid pair force (CalcForce2233, Source/Interaction.cpp:186-377) in
// FP32 with compensated sums. The FP64 preparation (prepare_wall_kernel:
// wall stress interpolation, partner-visible wall density, TIR) runs first;
// solid_copies32_kernel then takes the FP32 copies the pair loop reads.
// ---------------------------------------------------------------------------
// Symmetric 3x3 tensor (the stresses and TIR are symmetric: Jaumann rate of a
// symmetric stress, R diag R^T) as 6 floats in two float4: 00 01 02 11 | 12 22.
// An off-diagonal pair agrees to FP64 rounding (the two entries come from the
// same terms summed in another order), far below FP32's: the upper entry is
// taken. Conversions on the integer pipe (d2f_rn), no FP64 instruction.
PSPH_D void sym_store(float4* dst, size_t w, const double* m) {
  dst[2 * w] = make_float4(d2f_rn(m[0]), d2f_rn(m[1]), d2f_rn(m[2]), d2f_rn(m[4]));
  dst[2 * w + 1] = make_float4(d2f_rn(m[5]), d2f_rn(m[8]), 0.f, 0.f);
}

template <int DIM>
__global__ void __launch_bounds__(kFT32) solid_copies32_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= sc->n) return;
  const PClass32& C = v.cls32[P.cls[w]];
  if (v.inst[C.inst].stop) return;
  const double4_32a vv = P.V4[w];
  float lx, ly, lz;
  const float vx = d2f_split(vv.x, &lx), vy = d2f_split(vv.y, &ly), vz = d2f_split(vv.z, &lz);
  v.S.V32[w] = make_float4(vx, vy, vz, d2f_rn(vv.w));
  // the velocity's low-order part: near-rigid motion (a column settling as one
  // body) makes v_i - v_j far smaller than v, and the pair differences take
  // (hi_i - hi_j) + (lo_i - lo_j), exact to ~2^-48 of |v|
  v.S.V32LO[w] = make_float4(lx, ly, lz, 0.f);
  const double4_32a d = v.S.D4[w];
  v.S.D32[w] = make_float4(d2f_rn(d.x), d2f_rn(d.y), d2f_rn(d.z), d2f_rn(d.w));
  sym_store(v.S.SIG32, (size_t)w, P.sigma + 9 * (size_t)w);
  if (v.o.any_ti) sym_store(v.S.TIR32, (size_t)w, P.tir + 9 * (size_t)w);
  if (!(C.flags & CF_FREE)) {
    const double4_32a vb = (v.o.scheme == PSPH_MVERLET) ? P.H4[w] : P.H4b[w];
    v.S.VB32[w] = make_float4(d2f_rn(vb.x), d2f_rn(vb.y), d2f_rn(vb.z), 0.f);
    const double4_32a ns = v.S.nsv4[w];
    v.S.NSV32[w] = make_float4(d2f_rn(ns.x), d2f_rn(ns.y), d2f_rn(ns.z), 0.f);
  }
}

template <int DIM, int KT>
__global__ void __maxnreg__(128) forces_solid32_kernel(DevView v) {
  __shared__ double red[32];
  __shared__ unsigned long long cred[32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Options& o = v.o;
  const PClass32* __restrict__ CT = v.cls32;
  double dtc = DBL_MAX;
  unsigned npair2 = 0;  // 2 per pair with a free partner, 1 per wall partner (the pair is counted once)
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
  const float4 vil = v.S.V32LO[is];
  const float4 di4 = v.S.D32[is];
  const float di = di4.w, inv_i = di4.x, ci_snd = di4.z;
  const float mi = Ci.mass, hi = oi.w;
  const bool shep = (Ci.flags & CF_SHEPARD) && (Is.shepard_counter == o.shepard_step);
  const float4 sa = v.S.SIG32[2 * (size_t)is], sb = v.S.SIG32[2 * (size_t)is + 1];
  const float Si[6] = {sa.x, sa.y, sa.z, sa.w, sb.x, sb.y};
  float Ti[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (o.any_ti) {
    const float4 ta = v.S.TIR32[2 * (size_t)is], tb = v.S.TIR32[2 * (size_t)is + 1];
    Ti[0] = ta.x; Ti[1] = ta.y; Ti[2] = ta.z; Ti[3] = ta.w; Ti[4] = tb.x; Ti[5] = tb.y;
  }
  const float I22 = (DIM == 2) ? 0.f : 1.f;  // Domain::I (Source/Domain.cpp:1665)
  const float3 cs = cell_size_f(g);
  const bool xsph_on = o.xsph != 0.0;
  const float xsph = (float)o.xsph;
  const int grad_type = o.grad_type;
  Kahan ax, ay, az, dr;
  float zw = 0.f, sd = 0.f, xs0 = 0.f, xs1 = 0.f, xs2 = 0.f;
  float sr0 = 0.f, sr1 = 0.f, sr2 = 0.f, sr3 = 0.f, sr4 = 0.f, sr5 = 0.f;  // 00 01 02 11 12 22
  float rr0 = 0.f, rr1 = 0.f, rr2 = 0.f;                                  // 01 02 12
  const float cf2 = (float)(g.cellfac * g.cellfac);
  NbrSource<DIM> src;
  src.init(v, g, i, active && cell >= 0, 1.0f);
  while (true) {
    int code;
    const int j = src.next(v, &code);
    if (j < 0) break;
    const float4 oj = v.S.OFF32[j];
    float x0, x1, x2;
    rel_pos<DIM>(cs, oi, oj, code, x0, x1, x2);
    const float hb = 0.5f * (hi + oj.w);
    const float r2 = x0 * x0 + x1 * x1 + x2 * x2;
    if (r2 > cf2 * hb * hb) continue;  // the support test (the list holds a margin)
    const PClass32& Cj = CT[P.cls[j]];
    const int fjf = Cj.flags;
    const bool fj = fjf & CF_FREE;
    npair2 += fj ? 1ull : 2ull;
    const float ih = 1.f / hb;
    const float inv_r = (r2 > 0.f) ? rsqrtf(r2) : 0.f;
    const float q = r2 * inv_r * ih;
    const float ih2 = ih * ih;
    const float cwh = KernF<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * ih);
    const float cwg = cwh * ih2;
    const float GK = KernF<DIM, KT>::GK(q, hb * inv_r, cwg);
    const float K = KernF<DIM, KT>::W(q, cwh);
    const float4 vj = v.S.V32[j];
    const bool soil = (Ci.material * Cj.material == 9);
    float dj, inv_j, cj_snd = 0.f, mj;
    if (fj) {
      const float4 dj4 = v.S.D32[j];
      dj = dj4.w; inv_j = dj4.x; cj_snd = dj4.z; mj = Cj.mass;
    } else if (soil) {  // soil walls take the partner's density (Source/Interaction.cpp:201-205)
      dj = di; inv_j = inv_i; mj = Cj.fpmassc * mi;
    } else {
      if (o.uniform_eos) {
        const float4 dj4 = v.S.D32[j];
        dj = dj4.w; inv_j = dj4.x; cj_snd = dj4.z;
      } else {
        const PClass& C64 = v.cls[ci_cls];
        const double d64 = density_solid(C64.pres_eq, C64.cs, C64.p0, (double)vj.w, C64.rho0);
        dj = (float)d64;
        inv_j = 1.f / dj;
        cj_snd = (float)sound_speed(C64.pres_eq, C64.cs, d64, C64.rho0);
      }
      mj = Cj.fpmassc * mi;
    }
    const float4 vjl = v.S.V32LO[j];
    const float v0 = (vi.x - vj.x) + (vil.x - vjl.x), v1 = (vi.y - vj.y) + (vil.y - vjl.y),
                v2 = (vi.z - vj.z) + (vil.z - vjl.z);
    const float vx = v0 * x0 + v1 * x1 + v2 * x2;
    float PIs = 0.f;  // PIij = PIs I
    const float Alpha = 0.5f * (Ci.alpha + Cj.alpha), Beta = 0.5f * (Ci.beta + Cj.beta);
    if ((Alpha != 0.f || Beta != 0.f) && vx < 0.f) {
      const float Cij = soil ? 0.5f * (Ci.cs + Cj.cs) : 0.5f * (ci_snd + cj_snd);
      const float D = r2 + 0.01f * hb * hb;
      const float t = hb * vx;
      PIs = t * (Alpha * Cij * D + Beta * t) / (D * D * (0.5f * (di + dj)));
    }
    float vab0, vab1, vab2;
    if (fj) { vab0 = v0; vab1 = v1; vab2 = v2; }
    else if ((Ci.flags | fjf) & CF_NOSLIP) {
      const float4 ns = v.S.NSV32[j];
      vab0 = vi.x - (2.f * vj.x - ns.x);
      vab1 = vi.y - (2.f * vj.y - ns.y);
      vab2 = vi.z - (2.f * vj.z - ns.z);
    } else {
      const float4 vbj = v.S.VB32[j];
      vab0 = vi.x - vbj.x; vab1 = vi.y - vbj.y; vab2 = vi.z - vbj.z;
    }
    const float4 sja = v.S.SIG32[2 * (size_t)j], sjb = v.S.SIG32[2 * (size_t)j + 1];
    const float Sj[6] = {sja.x, sja.y, sja.z, sja.w, sjb.x, sjb.y};
    float M[6];
    if (grad_type == 0) {
      const float ci2 = inv_i * inv_i, cj2 = inv_j * inv_j;
#pragma unroll
      for (int e = 0; e < 6; ++e) M[e] = Si[e] * ci2 + Sj[e] * cj2;
    } else {
      const float c = inv_i * inv_j;
#pragma unroll
      for (int e = 0; e < 6; ++e) M[e] = (Si[e] + Sj[e]) * c;
    }
    M[0] += PIs; M[3] += PIs; M[5] += PIs * I22;
    if ((Ci.flags | fjf) & CF_TI) {
      const float Wd = KernF<DIM, KT>::W((Ci.tid + Cj.tid) * 0.5f * ih, cwh);
      const float TIs = powf(K / Wd, (Ci.tin + Cj.tin) * 0.5f);
      const float4 tja = v.S.TIR32[2 * (size_t)j], tjb = v.S.TIR32[2 * (size_t)j + 1];
      const float Tj[6] = {tja.x, tja.y, tja.z, tja.w, tjb.x, tjb.y};
#pragma unroll
      for (int e = 0; e < 6; ++e) M[e] += (Ti[e] + Tj[e]) * TIs;
    }
    const float g0 = GK * x0, g1 = GK * x1, g2 = GK * x2;
    // row vector (GK x_ij) times M (Mult, External/matvec.h:806)
    ax.add(mj * (g0 * M[0] + g1 * M[1] + g2 * M[2]));
    ay.add(mj * (g0 * M[1] + g1 * M[3] + g2 * M[4]));
    if (DIM == 3) az.add(mj * (g0 * M[2] + g1 * M[4] + g2 * M[5]));
    dr.add(mj * di * inv_j * (v0 * g0 + v1 * g1 + v2 * g2));
    const float md = mj * inv_j;
    zw += md * K;
    const float c2 = -0.5f * GK * md;
    sr0 += c2 * (2.f * vab0 * x0);
    sr1 += c2 * (vab0 * x1 + vab1 * x0);
    sr2 += c2 * (vab0 * x2 + vab2 * x0);
    sr3 += c2 * (2.f * vab1 * x1);
    sr4 += c2 * (vab1 * x2 + vab2 * x1);
    sr5 += c2 * (2.f * vab2 * x2);
    rr0 += c2 * (vab0 * x1 - vab1 * x0);
    rr1 += c2 * (vab0 * x2 - vab2 * x0);
    rr2 += c2 * (vab1 * x2 - vab2 * x1);
    if (xsph_on && fj) {
      const float s = xsph * mj / (0.5f * (di + dj)) * K;
      xs0 -= s * v0; xs1 -= s * v1; xs2 -= s * v2;
    }
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
    double* out = v.S.strain_rate + 9 * (size_t)i;
    out[0] = sr0; out[1] = sr1; out[2] = sr2;
    out[3] = sr1; out[4] = sr3; out[5] = sr4;
    out[6] = sr2; out[7] = sr4; out[8] = sr5;
    double* ro = v.S.rotation_rate + 9 * (size_t)i;
    ro[0] = 0.0; ro[1] = rr0; ro[2] = rr1;
    ro[3] = -(double)rr0; ro[4] = 0.0; ro[5] = rr2;
    ro[6] = -(double)rr1; ro[7] = -(double)rr2; ro[8] = 0.0;
    if (!(isfinite(axd) && isfinite(ayd) && isfinite(azd) && isfinite(drd))) atomicOr(&v.sc->status, ST_NONFINITE);
    // this particle's time-step bound sqrt_h_a sqrt(h/|a|) in FP32; the
    // minimum over particles and AdaptiveTimeStep stay FP64
    const float ax32 = (float)axd, ay32 = (float)ayd, az32 = (float)azd;
    const float an = sqrtf(ax32 * ax32 + ay32 * ay32 + az32 * az32);
    const double cand = (double)((float)o.sqrt_h_a * sqrtf(Ci.h / an));
    if (cand < dtc) dtc = cand;
  }
  block_dt_and_pairs<0>(v, Ci.inst, active, dtc, npair2, red, cred);
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
  const int bt = (v.o.pair_block >= 32 && v.o.pair_block <= kMaxPairBlock) ? v.o.pair_block : kFT32;
  const int nb = v.ncap <= 0 ? 1 : (v.ncap + bt - 1) / bt;
  if (v.o.has_solid) {
    switch (v.o.kt) {
      case 0: forces_solid32_kernel<DIM, 0><<<nb, bt, 0, st>>>(v); break;
      case 1: forces_solid32_kernel<DIM, 1><<<nb, bt, 0, st>>>(v); break;
      default: forces_solid32_kernel<DIM, 2><<<nb, bt, 0, st>>>(v); break;
    }
    return;
  }
  const Options& o = v.o;
  const bool spec = o.vis_eq == 0 && o.grad_type == 0 && !o.any_ti && o.xsph == 0.0 && o.uniform_h &&
                    o.uniform_av && o.uniform_mass && (o.uniform_mu || o.dyn_mu);
  const int fl = spec ? (o.need_sr ? (o.closure ? 3 : 2) : 1) : 0;
  switch (o.kt * 4 + fl) {
    case 0: forces_fluid32_kernel<DIM, 0, 0><<<nb, bt, 0, st>>>(v); break;
    case 1: forces_fluid32_kernel<DIM, 0, 1><<<nb, bt, 0, st>>>(v); break;
    case 2: forces_fluid32_kernel<DIM, 0, 2><<<nb, bt, 0, st>>>(v); break;
    case 3: forces_fluid32_kernel<DIM, 0, 3><<<nb, bt, 0, st>>>(v); break;
    case 4: forces_fluid32_kernel<DIM, 1, 0><<<nb, bt, 0, st>>>(v); break;
    case 5: forces_fluid32_kernel<DIM, 1, 1><<<nb, bt, 0, st>>>(v); break;
    case 6: forces_fluid32_kernel<DIM, 1, 2><<<nb, bt, 0, st>>>(v); break;
    case 7: forces_fluid32_kernel<DIM, 1, 3><<<nb, bt, 0, st>>>(v); break;
    case 8: forces_fluid32_kernel<DIM, 2, 0><<<nb, bt, 0, st>>>(v); break;
    case 9: forces_fluid32_kernel<DIM, 2, 1><<<nb, bt, 0, st>>>(v); break;
    case 10: forces_fluid32_kernel<DIM, 2, 2><<<nb, bt, 0, st>>>(v); break;
    default: forces_fluid32_kernel<DIM, 2, 3><<<nb, bt, 0, st>>>(v); break;
  }
}

}  // namespace

void launch_prepare32(const DevView& v, cudaStream_t st) {
  if (v.o.has_solid) {  // FP64 wall stress interpolation and TIR, then the FP32 copies
    launch_prepare(v, st);
    const int nb = nblk32(v.ncap);
    if (v.o.dim == 2) solid_copies32_kernel<2><<<nb, kFT32, 0, st>>>(v);
    else solid_copies32_kernel<3><<<nb, kFT32, 0, st>>>(v);
    return;
  }
  if (v.o.dim == 2) prepare32_dispatch<2>(v, st);
  else prepare32_dispatch<3>(v, st);
}

namespace {
__global__ void expand_sr32_kernel(const float* __restrict__ sr32, double* __restrict__ sr, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* a = sr32 + 6 * (size_t)i;
  double* o = sr + 9 * (size_t)i;
  o[0] = a[0]; o[1] = a[1]; o[2] = a[2];
  o[3] = a[1]; o[4] = a[3]; o[5] = a[4];
  o[6] = a[2]; o[7] = a[4]; o[8] = a[5];
}
}  // namespace

void launch_expand_sr32(const DevView& v, int n, cudaStream_t st) {
  if (n > 0 && v.S.sr32 && v.S.strain_rate)
    expand_sr32_kernel<<<(n + 255) / 256, 256, 0, st>>>(v.S.sr32, v.S.strain_rate, n);
}

void launch_forces32(const DevView& v, cudaStream_t st) {
  if (v.o.dim == 2) forces32_dispatch<2>(v, st);
  else forces32_dispatch<3>(v, st);
}

}  // namespace psph
