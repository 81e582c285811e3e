// Gather-form pair kernels of the GB300 hot path.
//
// The reference walks a half stencil of cells, pushes every candidate pair into
// per-thread lists and then scatters each pair's contribution into both
// particles under per-particle locks (Source/Domain.cpp:808-945,
// Source/Interaction.cpp:25-377). Here each particle gathers from the full
// 3x3(x3) block of cells around its own, so every pair is evaluated twice (once
// from each side) and each particle's sums are owned by one thread: no atomics,
// no locks, deterministic results.
//
//   prepare_wall  free particles: partner-visible density / sound speed, TIR;
//                 fixed particles: PrimaryComputeAcceleration's wall
//                 interpolation (Source/Domain.cpp:1020-1059, :1164-1206)
//   forces_fluid  CalcForce11 (Source/Interaction.cpp:25-184) from the side of
//                 each free particle, plus the acceleration time-step bound
//   forces_solid  CalcForce2233 (Source/Interaction.cpp:186-377)
//   dt_finalize   LastComputeAcceleration's minimum (Source/Domain.cpp:1280-1296)
//                 and AdaptiveTimeStep (Source/Domain.cpp:133-152)
#include <cfloat>

#include "psph_pairs.cuh"

namespace psph {

namespace {

constexpr int kFT = 128;  // threads per block of the pair kernels

template <int DIM>
PSPH_D void tensile_tir(const double* S, double TI, double rho, double* TIR) {
  // Source/Domain.cpp:958-976 (2D); 3D via a Jacobi eigen-decomposition
  // (the reference uses GSL's symmetric eigensolver, :979-987).
  // No principal stress in tension (the usual state of a soil column): the
  // reference's R diag(0) R^T is zero. The bound is conservative by 1e-12 of
  // the stress scale, far above the rounding of either eigen-decomposition,
  // and skips the FP64 trigonometry or Jacobi sweeps for these particles.
  // The same bound first in FP32 from truncated copies (integer pipe, no FP64
  // square root): their errors stay below ~1e-6 of the scale, so an FP32
  // bound under -1e-5 of the scale implies the exact test below.
  {
    float bound, scale;
    const float s0 = d2f_bits(S[0]), s1 = d2f_bits(S[1]), s4 = d2f_bits(S[4]);
    if (DIM == 2) {
      const float m = 0.5f * (s0 + s4), d = 0.5f * (s0 - s4);
      bound = m + sqrtf(d * d + s1 * s1);
      scale = fabsf(s0) + fabsf(s4) + fabsf(s1);
    } else {
      const float s2 = d2f_bits(S[2]), s3 = d2f_bits(S[3]), s5 = d2f_bits(S[5]);
      const float s6 = d2f_bits(S[6]), s7 = d2f_bits(S[7]), s8 = d2f_bits(S[8]);
      bound = fmaxf(s0 + fabsf(s1) + fabsf(s2), fmaxf(s4 + fabsf(s3) + fabsf(s5), s8 + fabsf(s6) + fabsf(s7)));
      scale = fabsf(s0) + fabsf(s4) + fabsf(s8) + fabsf(s1) + fabsf(s2) + fabsf(s5);
    }
    if (bound < -1e-5f * scale) {
      if (DIM == 2) TIR[0] = TIR[1] = TIR[3] = TIR[4] = 0.0;
      else
        for (int e = 0; e < 9; ++e) TIR[e] = 0.0;
      return;
    }
  }
  {
    double bound, scale;
    if (DIM == 2) {
      const double m = 0.5 * (S[0] + S[4]), d = 0.5 * (S[0] - S[4]);
      bound = m + sqrt(d * d + S[1] * S[1]);  // the larger in-plane eigenvalue
      scale = fabs(S[0]) + fabs(S[4]) + fabs(S[1]);
    } else {  // Gershgorin: every eigenvalue is below the largest row bound
      const double r0 = S[0] + fabs(S[1]) + fabs(S[2]);
      const double r1 = S[4] + fabs(S[3]) + fabs(S[5]);
      const double r2 = S[8] + fabs(S[6]) + fabs(S[7]);
      bound = fmax(r0, fmax(r1, r2));
      scale = fabs(S[0]) + fabs(S[4]) + fabs(S[8]) + fabs(S[1]) + fabs(S[2]) + fabs(S[5]);
    }
    if (bound < -1e-12 * scale) {
      if (DIM == 2) TIR[0] = TIR[1] = TIR[3] = TIR[4] = 0.0;  // the entries the 2D rotation writes
      else
        for (int e = 0; e < 9; ++e) TIR[e] = 0.0;
      return;
    }
  }
  if (DIM == 2) {
    double teta;
    if ((S[0] - S[4]) != 0.0) teta = 0.5 * atan(2.0 * S[1] / (S[0] - S[4]));
    else teta = kPi / 4.0;
    const double C = cos(teta), Sn = sin(teta);
    double Sxx = C * C * S[0] + 2.0 * C * Sn * S[1] + Sn * Sn * S[4];
    double Syy = Sn * Sn * S[0] - 2.0 * C * Sn * S[1] + C * C * S[4];
    Sxx = (Sxx > 0) ? -TI * Sxx / (rho * rho) : 0.0;
    Syy = (Syy > 0) ? -TI * Syy / (rho * rho) : 0.0;
    TIR[0] = C * C * Sxx + Sn * Sn * Syy;
    TIR[4] = Sn * Sn * Sxx + C * C * Syy;
    TIR[1] = TIR[3] = Sn * C * (Sxx - Syy);
  } else {
    double a[9], Q[9];
    for (int e = 0; e < 9; ++e) {
      a[e] = S[e];
      Q[e] = (e % 4 == 0) ? 1.0 : 0.0;
    }
    for (int sweep = 0; sweep < 50; ++sweep) {
      if (a[1] * a[1] + a[2] * a[2] + a[5] * a[5] == 0.0) break;
      for (int p = 0; p < 3; ++p)
        for (int r = p + 1; r < 3; ++r) {
          const double apr = a[3 * p + r];
          if (apr == 0.0) continue;
          const double theta = (a[3 * r + r] - a[3 * p + p]) / (2.0 * apr);
          const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
          const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
          for (int k = 0; k < 3; ++k) {
            const double akp = a[3 * k + p], akr = a[3 * k + r];
            a[3 * k + p] = c * akp - s * akr;
            a[3 * k + r] = s * akp + c * akr;
          }
          for (int k = 0; k < 3; ++k) {
            const double apk = a[3 * p + k], ark = a[3 * r + k];
            a[3 * p + k] = c * apk - s * ark;
            a[3 * r + k] = s * apk + c * ark;
          }
          for (int k = 0; k < 3; ++k) {
            const double qkp = Q[3 * k + p], qkr = Q[3 * k + r];
            Q[3 * k + p] = c * qkp - s * qkr;
            Q[3 * k + r] = s * qkp + c * qkr;
          }
        }
    }
    double val[3];
    for (int k = 0; k < 3; ++k) {
      const double ev = a[4 * k];
      val[k] = (ev > 0) ? -TI * ev / (rho * rho) : 0.0;
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) TIR[3 * r + c] = Q[3 * r + 0] * val[0] * Q[3 * c + 0] + Q[3 * r + 1] * val[1] * Q[3 * c + 1] + Q[3 * r + 2] * val[2] * Q[3 * c + 2];
  }
}
constexpr int kQN = 16;  // queued FP64 pair evaluations per lane between flushes

// ---------------------------------------------------------------------------
// Per-particle preparation and wall interpolation
// ---------------------------------------------------------------------------
template <int DIM, int KT>
__global__ void __launch_bounds__(kFT) prepare_wall_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const Options& o = v.o;
  const PClass* __restrict__ CT = v.cls;
  const int winst = (w < n) ? CT[P.cls[w]].inst : 0;
  const GridDev& g = grid_of(v, winst);
  const bool run = (w < n) && !v.inst[winst].stop;
  bool wall = false;
  int mat = 0;
  double sk = 0.0, p = 0.0, n0 = 0.0, n1 = 0.0, n2 = 0.0;
  double sig[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) sig[e] = 0.0;
  double4_32a xw = make_double4_32a(0, 0, 0, 0);
  int ow = 0, cell = -1;
  double hw = 0.0;
  bool noslip = false;
  if (run) {
    const PClass& Cw = CT[P.cls[w]];
    if (Cw.is_free) {
      const double rho = P.X4[w].w;
      const double inv = 1.0 / rho;
      const double pr = P.V4[w].w;
      v.S.D4[w] = make_double4_32a(inv, pr * inv * inv, sound_speed(Cw.pres_eq, Cw.cs, rho, Cw.rho0), rho);
      if (o.has_solid && Cw.material > 1 && Cw.ti > 0.0)
        tensile_tir<DIM>(P.sigma + 9 * (size_t)w, Cw.ti, rho, P.tir + 9 * (size_t)w);
    } else {
      wall = true;
      mat = Cw.material;
      xw = P.X4[w];
      ow = P.orig[w];
      cell = v.S.cellid[w];
      hw = Cw.h;
      noslip = Cw.no_slip;
    }
  }
  // Wall interpolation (FSMPairs only: free partners of the same material).
  const bool any_periodic = g.periodic[0] | g.periodic[1] | g.periodic[2];
  const double gx = o.gravity[0], gy = o.gravity[1], gz = o.gravity[2];
  const bool need_orient = !o.wallp_physical && (gx != 0.0 || gy != 0.0 || gz != 0.0) && mat < 3;
  const CellCoord cw = decode(g, cell >= 0 ? cell : 0);
  // one neighbour (a free particle of the same material contributes): its
  // position and velocity loads go out with its class, ahead of the class test
  auto visit = [&](const int f, const int fcode) {
    const int clsf = P.cls[f];
    const double4_32a xf = P.X4[f];
    const double4_32a vf = P.V4[f];
    const PClass& Cf = CT[clsf];
    if (!Cf.is_free || Cf.material != mat) return;
    const double hb = (hw + Cf.h) / 2.0;
    CellCoord cf = cw;
    if (any_periodic) cf = decode(g, v.S.cellid[f]);
    const bool wfirst = need_orient ? first_of_pair_code(fcode, ow, P.orig[f]) : true;
    double x0, x1, x2;
    if (wfirst) {
      x0 = xw.x - xf.x; x1 = xw.y - xf.y; x2 = xw.z - xf.z;
      if (any_periodic) periodic_fix(g, x0, x1, x2, hb, cw, cf);
    } else {
      x0 = xf.x - xw.x; x1 = xf.y - xw.y; x2 = xf.z - xw.z;
      if (any_periodic) periodic_fix(g, x0, x1, x2, hb, cf, cw);
    }
    const double r = sqrt(x0 * x0 + x1 * x1 + x2 * x2);
    const double inv_hb = o.uniform_h ? o.inv_h : 1.0 / hb;
    const double q = r * inv_hb;
    const double ih2 = inv_hb * inv_hb;
    const double K = Kern<DIM, KT>::W(q, Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_hb));
    if (K == 0.0) return;
    sk += K;
    if (mat < 3) p += vf.w * K + (gx * x0 + gy * x1 + gz * x2) * xf.w * K;
    if (mat > 1) {
      const double* sf = P.sigma + 9 * (size_t)f;
#pragma unroll
      for (int e = 0; e < 9; ++e) sig[e] += sf[e] * K;
    }
    if (noslip) { n0 += vf.x * K; n1 += vf.y * K; n2 += vf.z * K; }
  };
  const int cnt = (wall && cell >= 0) ? v.S.nl_count[w] : 0;
  if (cnt >= 0) {  // the neighbour list, 4 entries per 16-byte load
    const int4* __restrict__ nl4 = reinterpret_cast<const int4*>(v.S.nl) + nl_slot(w);
    const size_t N = (size_t)v.nl_stride;
    const int nch = (cnt + 3) >> 2;
    for (int ch = 0; ch < nch; ++ch) {
      const int4 qe = nl4[(size_t)ch * N];
      const int rem = cnt - 4 * ch;
      visit(qe.x & kIndexMask, qe.x >> kCodeShift);
      if (rem > 1) visit(qe.y & kIndexMask, qe.y >> kCodeShift);
      if (rem > 2) visit(qe.z & kIndexMask, qe.z >> kCodeShift);
      if (rem > 3) visit(qe.w & kIndexMask, qe.w >> kCodeShift);
    }
  } else {  // list overflow: scan the cells
    NbrSource<DIM> src;
    src.init(v, g, w, true, 1.004f);
    while (true) {
      int code;
      const int f = src.next(v, &code);
      if (f < 0) break;
      visit(f, code);
    }
  }
  if (!wall) return;
  const PClass& Cw = CT[P.cls[w]];
  const PClass& Ce = CT[o.eos_cls];
  if (sk != 0.0) {
    if (mat < 3) p = p / sk;
    if (mat > 1) {
      const double s = 1.0 / sk;
#pragma unroll
      for (int e = 0; e < 9; ++e) sig[e] = sig[e] * s;
    }
    if (noslip) { n0 = n0 / sk; n1 = n1 / sk; n2 = n2 / sk; }
  } else {
    p = 0.0; n0 = n1 = n2 = 0.0;
  }
  double4_32a vw = P.V4[w];
  vw.w = p;
  P.V4[w] = vw;
  v.S.sumkernel[w] = sk;
  v.S.nsv4[w] = make_double4_32a(n0, n1, n2, 0.0);
  if (o.has_solid) {
    double* sw = P.sigma + 9 * (size_t)w;
#pragma unroll
    for (int e = 0; e < 9; ++e) sw[e] = sig[e];
    if (P.shear) {
      double* tw = P.shear + 9 * (size_t)w;
#pragma unroll
      for (int e = 0; e < 9; ++e) tw[e] = 0.0;
    }
    if (sk != 0.0 && mat > 1 && Cw.ti > 0.0) tensile_tir<DIM>(sig, Cw.ti, xw.w, P.tir + 9 * (size_t)w);
  }
  // density, 1/density, p/density^2 and sound speed the partners see (Source/Interaction.cpp:41-61)
  double rw = xw.w, cwv = 0.0;
  if (o.uniform_eos && mat != 3) {
    rw = density_solid(Ce.pres_eq, Ce.cs, Ce.p0, p, Ce.rho0);
    cwv = sound_speed(Ce.pres_eq, Ce.cs, rw, Ce.rho0);
  }
  const double inv = 1.0 / rw;
  v.S.D4[w] = make_double4_32a(inv, p * inv * inv, cwv, rw);
}

// ---------------------------------------------------------------------------
// Fluid pair force (CalcForce11) from the side of free particle i.
//
// HALF = false: every pair is evaluated from both sides (the gather form).
// HALF = true (pass A of the once-per-pair form): CalcForce11 updates both
// particles of a pair from one evaluation (Source/Interaction.cpp:139-145), so
// a pair of two free particles whose neighbour lists are both in use is
// evaluated once, by one side (evaluates_pair), which keeps its own terms and
// writes the partner's terms (a, dDensity, ZWab, SumDen) into the partner's
// own list slot of the pair: each list ascends as unsigned (cell-offset code
// << 26 | index), so the partner's entry for i is found by a binary search
// for (mirror code, i). Pairs with a wall are evaluated by the free side, as
// in the gather form. forces_fluid_fold_kernel (pass B) then adds the
// partners' terms in list order. Both sums keep a fixed order: no atomics,
// deterministic results.
// ---------------------------------------------------------------------------
// Which side of a shared pair evaluates it: by the parity of i + j the lower or
// the higher index, so each particle evaluates about half of its shared pairs
// whatever its place in its cell (the lanes of a warp then carry nearly equal
// queues); own(i, j) == !own(j, i) for i != j.
PSPH_D bool evaluates_pair(int i, int j) { return ((i ^ j) & 1) ? (i < j) : (i > j); }

// i's slot in j's list: the entry (mirror code, i) of j's ascending list, or -1
PSPH_D int partner_slot(const DevView& v, int j, int code, int i) {
  const unsigned key = ((unsigned)(26 - code) << kCodeShift) | (unsigned)i;
  int lo = 0, hi = v.S.nl_count[j] - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const unsigned e = (unsigned)v.S.nl[nl_index(v.nl_stride, j, mid)];
    if (e == key) return mid;
    if (e < key) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

template <int DIM, int KT, bool HALF>
__global__ void __launch_bounds__(kFT) forces_fluid_kernel(DevView v) {
  __shared__ double red[kFT / 32];
  __shared__ unsigned long long cred[kFT / 32];
  __shared__ int qbuf[kQN][kFT];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int tid = threadIdx.x;
  const Options& o = v.o;
  const PClass* __restrict__ CT = v.cls;
  double dtc = DBL_MAX;
  unsigned long long npair2 = 0;
  bool active = false;
  int cell = -1, ci_cls = 0;
  if (i < n) {
    ci_cls = P.cls[i];
    // a domain of two materials runs this kernel for its fluid particles only
    const bool run = !v.inst[CT[ci_cls].inst].stop && (!o.mixed || CT[ci_cls].material == 1);
    active = run && CT[ci_cls].is_free;
    cell = v.S.cellid[i];
    if (run && !active) {
      if (!o.a_from_hook) v.S.A4[i] = make_double4_32a(o.gravity[0], o.gravity[1], o.gravity[2], 0.0);
      v.S.zwab[i] = 1.0;
      if (v.S.s_acc) v.S.s_acc[i] = 0.0;
    }
  }
  const PClass& Ci = CT[ci_cls];
  const GridDev& g = grid_of(v, Ci.inst);
  const InstState& Is = v.inst[Ci.inst];
  const double4_32a xi = active ? P.X4[i] : make_double4_32a(0, 0, 0, 1);
  const double4_32a vi = active ? P.V4[i] : make_double4_32a(0, 0, 0, 0);
  const double4_32a di4 = active ? v.S.D4[i] : make_double4_32a(1, 0, 0, 1);
  const double di = xi.w, inv_i = di4.x, Pi = di4.y, ci_snd = di4.z, pi = vi.w;
  const double mi = Ci.mass, hi = Ci.h;
  const double mui = o.dyn_mu ? (active ? P.mu[i] : 0.0) : Ci.mu0;
  const bool shep = Ci.shepard && (Is.shepard_counter == o.shepard_step);
  const bool sr_self = (Ci.t0 > 0.0 || Ci.les);
  double ax = o.gravity[0] + o.body_force[0], ay = o.gravity[1] + o.body_force[1],
         az = o.gravity[2] + o.body_force[2];
  double drho = 0.0, zw = 0.0, sd = 0.0, xs0 = 0.0, xs1 = 0.0, xs2 = 0.0;
  if (o.a_from_hook && active) {  // StartAcceleration's values as a GeneralBefore hook left them
    const double4_32a a0 = v.S.A4[i];
    ax = a0.x + o.body_force[0];
    ay = a0.y + o.body_force[1];
    az = a0.z + o.body_force[2];
    drho = a0.w;
  }
  double sr0 = 0.0, sr1 = 0.0, sr2 = 0.0, sr4 = 0.0, sr5 = 0.0, sr8 = 0.0;
  double w01 = 0.0, w02 = 0.0, w12 = 0.0;  // antisymmetric counterpart of the strain-rate sums (closure)
  double ss = 0.0;  // SWIType 1: the surface-erosion velocity derivative S
  const bool want_s = v.S.s_acc != nullptr;
  int nnb = 0;
  const bool closure = o.closure && Ci.les;
  const bool any_periodic = g.periodic[0] | g.periodic[1] | g.periodic[2];
  CellCoord cci = decode(g, cell >= 0 ? cell : 0);
  NbrSource<DIM> src;
  src.init(v, g, i, active && cell >= 0, 1.004f);
  bool more = active && cell >= 0;
  // once-per-pair form: i's list is in use (not overflowed)
  const bool own_list = HALF && active && cell >= 0 && v.S.nl_count[i] >= 0;
  const int shep_pair = o.shepard_step;  // the counter is per instance: partners share it
  // a partner slot written this step carries the instance's step number + 1
  const int stamp = (int)(Is.steps & 0x3fffffff) + 1;
  while (true) {
    int qn = 0;
    while (more && qn < kQN) {
      int code;
      const int j = src.next(v, &code);
      if (j < 0) {
        more = false;
        break;
      }
      // once-per-pair form: a shared pair the partner evaluates is left out of
      // the queue, so the lanes' queues hold only work
      if (HALF && own_list && !evaluates_pair(i, j) && v.S.nl_count[j] >= 0 && CT[P.cls[j]].is_free) continue;
      qbuf[qn++][tid] = HALF ? (j | (code << kCodeShift)) : j;
    }
    const int qmax = __reduce_max_sync(0xffffffffu, qn);
    for (int k = 0; k < qmax; ++k) {
      if (k >= qn) continue;
      const int qe = qbuf[k][tid];
      const int j = HALF ? (qe & kIndexMask) : qe;
      const double4_32a xj = P.X4[j];
      const PClass& Cj = CT[P.cls[j]];
      if (!HALF && o.mixed && Cj.material != 1) continue;  // soil or solid partners: the coupling kernel
      // shared pair: both free, both lists in use; evaluates_pair picks the
      // side (the queue holds only those this side evaluates)
      const bool share = own_list && Cj.is_free && v.S.nl_count[j] >= 0;
      const double hb = (hi + Cj.h) / 2;
      double x0 = xi.x - xj.x, x1 = xi.y - xj.y, x2 = xi.z - xj.z;
      if (any_periodic) periodic_fix(g, x0, x1, x2, hb, cci, decode(g, v.S.cellid[j]));
      const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
      const double inv_hb = o.uniform_h ? o.inv_h : 1.0 / hb;
      double rij, inv_r = 0.0;
      if (KT == 1 && o.vis_eq <= 1) {
        rij = sqrt(r2);
      } else {
        inv_r = (r2 > 0.0) ? rsqrt(r2) : 0.0;
        rij = r2 * inv_r;
      }
      const double q = rij * inv_hb;
      if (q > g.cellfac) continue;
      const bool fj = Cj.is_free;
      npair2 += fj ? 1ull : 2ull;
      ++nnb;
      const double4_32a vj = P.V4[j];
      const double4_32a dj4 = v.S.D4[j];
      double dj, inv_j, Pj, cj_snd;
      const double mj = fj ? Cj.mass : Cj.fpmassc * mi;
      const double pj = vj.w;
      if (fj || o.uniform_eos) {
        dj = dj4.w; inv_j = dj4.x; Pj = dj4.y; cj_snd = dj4.z;
      } else {  // wall density from this particle's EOS (Source/Interaction.cpp:53-57)
        dj = density_solid(Ci.pres_eq, Ci.cs, Ci.p0, pj, Ci.rho0);
        inv_j = 1.0 / dj;
        Pj = pj * inv_j * inv_j;
        cj_snd = sound_speed(Ci.pres_eq, Ci.cs, dj, Ci.rho0);
      }
      const double ih2 = inv_hb * inv_hb;
      const double cwh = Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_hb);
      const double cwg = cwh * ih2;
      const double inv_q = hb * inv_r;
      const double GK = Kern<DIM, KT>::GK(q, inv_q, cwg);
      const double K = Kern<DIM, KT>::W(q, cwh);
      const double v0 = vi.x - vj.x, v1 = vi.y - vj.y, v2 = vi.z - vj.z;
      const double vx = v0 * x0 + v1 * x1 + v2 * x2;
      double PI = 0.0;
      const double Alpha = (Ci.alpha + Cj.alpha) / 2.0, Beta = (Ci.beta + Cj.beta) / 2.0;
      if ((Alpha != 0.0 || Beta != 0.0) && vx < 0) {
        // (-a c MU + b MU^2) / rho_ij with MU = h v.x / D, as one division
        const double D = r2 + 0.01 * hb * hb;
        const double t = hb * vx;
        PI = t * (-Alpha * 0.5 * (ci_snd + cj_snd) * D + Beta * t) / (D * D * (0.5 * (di + dj)));
      }
      double TI = 0.0;
      if (Ci.ti > 0.0 || Cj.ti > 0.0) {
        double Ri = 0.0, Rj = 0.0;
        if ((pi + pj) < 0.0) {
          if (pi < 0.0) Ri = -pi * inv_i * inv_i;
          if (pj < 0.0) Rj = -pj * inv_j * inv_j;
        }
        const double Wd = Kern<DIM, KT>::W((Ci.tid + Cj.tid) / (2.0 * hb), cwh);
        TI = (Ci.ti * Ri + Cj.ti * Rj) * pow(K / Wd, (Ci.tin + Cj.tin) / 2.0);
      }
      double VI0 = 0.0, VI1 = 0.0, VI2 = 0.0;
      double vab0 = 0.0;
      if ((Ci.no_slip || Cj.no_slip) || fj) {
        double Mu, vab1, vab2;
        if (fj) {
          vab0 = v0; vab1 = v1; vab2 = v2;
          if (o.uniform_mu) Mu = o.mu_u;
          else {
            const double muj = o.dyn_mu ? P.mu[j] : Cj.mu0;
            Mu = 2.0 * mui * muj / (mui + muj);
          }
        } else {
          const double4_32a ns = v.S.nsv4[j];
          vab0 = vi.x - (2.0 * vj.x - ns.x);
          vab1 = vi.y - (2.0 * vj.y - ns.y);
          vab2 = vi.z - (2.0 * vj.z - ns.z);
          Mu = mui;
        }
        if (o.vis_eq <= 2) {
          double c;
          if (o.vis_eq == 0) c = 2.0 * Mu * inv_i * inv_j * GK;
          else if (o.vis_eq == 1) c = 8.0 * Mu / ((di + dj) * (di + dj)) * GK;
          else c = -Mu * inv_i * inv_j * Kern<DIM, KT>::Lap(q, inv_q, cwg);
          VI0 = c * vab0; VI1 = c * vab1; VI2 = c * vab2;
        } else {
          const double L = Kern<DIM, KT>::Lap(q, inv_q, cwg);
          const double S2 = Kern<DIM, KT>::D2(q, cwg);
          const double s = -Mu * inv_i * inv_j;
          const double t = vx / r2 * (-GK + S2);
          VI0 = s * (L * vab0 + (1.0 / 3.0) * (GK * v0 + t * x0));
          VI1 = s * (L * vab1 + (1.0 / 3.0) * (GK * v1 + t * x1));
          VI2 = s * (L * vab2 + (1.0 / 3.0) * (GK * v2 + t * x2));
        }
        if (sr_self && (Ci.t0 > 0.0 || Cj.t0 > 0.0 || (Ci.les && Cj.les))) {
          const double c2 = -GK * (mj * inv_j);
          sr0 += c2 * (2.0 * vab0 * x0);
          sr1 += c2 * (vab0 * x1 + vab1 * x0);
          sr2 += c2 * (vab0 * x2 + vab2 * x0);
          sr4 += c2 * (2.0 * vab1 * x1);
          sr5 += c2 * (vab1 * x2 + vab2 * x1);
          sr8 += c2 * (2.0 * vab2 * x2);
          if (closure) {
            w01 += c2 * (vab0 * x1 - vab1 * x0);
            w02 += c2 * (vab0 * x2 - vab2 * x0);
            w12 += c2 * (vab1 * x2 - vab2 * x1);
          }
        }
      }
      if (o.xsph != 0.0 && fj) {
        const double s = o.xsph * mj / (0.5 * (di + dj)) * K;
        xs0 -= s * v0; xs1 -= s * v1; xs2 -= s * v2;
      }
      double s;
      if (o.grad_type == 0) s = -(Pi + Pj + PI + TI) * GK;
      else s = -((pi + pj) * inv_i * inv_j + PI + TI) * GK;
      ax += mj * (s * x0 + VI0);
      ay += mj * (s * x1 + VI1);
      if (DIM == 3) az += mj * (s * x2 + VI2);
      drho += mj * di * inv_j * (GK * vx);
      zw += mj * inv_j * K;
      if (shep) sd += mj * K;
      if (!HALF && want_s) ss = ss + mj / dj * vab0 * x1 * -GK;  // Source/Interaction.cpp:154
      if (HALF && share) {
        // j's terms of this evaluation, seen from j (x_ji = -x_ij, v_ji = -v_ij):
        // a_j -= m_i F, dDensity_j += m_i (rho_j / rho_i) v.GK x, ZWab_j += m_i / rho_i W,
        // SumDen_j += m_i W (Source/Interaction.cpp:139-145, :170-177)
        npair2 += 1ull;  // the partner's half of the count
        const int slot = partner_slot(v, j, qe >> kCodeShift, i);
        if (slot < 0) {
          atomicOr(&v.sc->status, ST_LIST_MISMATCH);
        } else {
          const size_t e = nl_index(v.nl_stride, j, slot);
          const double fx = mi * (s * x0 + VI0), fy = mi * (s * x1 + VI1), fz = DIM == 3 ? mi * (s * x2 + VI2) : 0.0;
          v.S.half4[e] = make_double4_32a(-fx, -fy, -fz, mi * dj * inv_i * (GK * vx));
          const bool shep_j = Cj.shepard && (Is.shepard_counter == shep_pair);
          v.S.half2[e] = make_double2(mi * inv_i * K, shep_j ? mi * K : 0.0);
          v.S.half_stamp[e] = stamp;  // written this step
        }
      }
    }
    if (!__any_sync(0xffffffffu, more)) break;
  }
  if (HALF) {  // own terms; pass B adds the partners', then the dt bound
    if (active) {
      v.S.A4[i] = make_double4_32a(ax, ay, az, drho);
      v.S.zwab[i] = zw;
      if (o.any_shepard) v.S.sumden[i] = sd;
    }
    block_dt_and_pairs<kFT>(v, Ci.inst, false, dtc, npair2, red, cred);
    return;
  }
  if (active) {
    v.S.A4[i] = make_double4_32a(ax, ay, az, drho);
    v.S.zwab[i] = zw;
    if (o.any_shepard) v.S.sumden[i] = sd;
    if (want_s) v.S.s_acc[i] = ss;
    if (o.xsph != 0.0) v.S.vxsph4[i] = make_double4_32a(xs0, xs1, xs2, 0.0);
    if (o.need_sr) {
      double* out = v.S.strain_rate + 9 * (size_t)i;
      out[0] = sr0; out[1] = sr1; out[2] = sr2;
      out[3] = sr1; out[4] = sr4; out[5] = sr5;
      out[6] = sr2; out[7] = sr5; out[8] = sr8;
    }
    if (closure) {
      v.S.cvort[i] = (float)sqrt(w01 * w01 + w02 * w02 + w12 * w12);
      v.S.cnnb[i] = (float)nnb;
    }
    if (!(isfinite(ax) && isfinite(ay) && isfinite(az) && isfinite(drho))) atomicOr(&v.sc->status, ST_NONFINITE);
    const double an = sqrt(ax * ax + ay * ay + az * az);
    const double cand = o.sqrt_h_a * sqrt(hi / an);
    if (cand < dtc) dtc = cand;  // NaN never compares less, as in the reference
  }
  // two materials: the dt bound waits for the coupling kernel's terms
  block_dt_and_pairs<kFT>(v, Ci.inst, active && !o.mixed, dtc, npair2, red, cred);
}

// Pass B of the once-per-pair form: adds, in list order, the terms the
// partners that evaluated their pair wrote into i's slots this step (their slot
// stamp is this step's; a slot of a pair outside the support, or of a partner
// that evaluated its own side, keeps an older stamp), then the dt bound and
// the finiteness check of the gather form.
template <int DIM>
__global__ void __launch_bounds__(kFT) forces_fluid_fold_kernel(DevView v) {
  __shared__ double red[kFT / 32];
  __shared__ unsigned long long cred[kFT / 32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Options& o = v.o;
  const PClass* __restrict__ CT = v.cls;
  bool active = false;
  int cell = -1, ci_cls = 0;
  if (i < n) {
    ci_cls = P.cls[i];
    active = !v.inst[CT[ci_cls].inst].stop && CT[ci_cls].is_free;
    cell = v.S.cellid[i];
  }
  const PClass& Ci = CT[ci_cls];
  double dtc = DBL_MAX;
  if (active) {
    const int stamp = (int)(v.inst[Ci.inst].steps & 0x3fffffff) + 1;
    double4_32a a = v.S.A4[i];
    double zw = v.S.zwab[i], sd = o.any_shepard ? v.S.sumden[i] : 0.0;
    const int cnt = cell >= 0 ? v.S.nl_count[i] : -1;
    const int4* __restrict__ nl4 = reinterpret_cast<const int4*>(v.S.nl) + nl_slot(i);
    const size_t N = (size_t)v.nl_stride;
    for (int c = 0; 4 * c < cnt; ++c) {  // one 16-byte chunk of 4 entries per load
      const int4 q = nl4[(size_t)c * N];
      const int ent[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (4 * c + e >= cnt || evaluates_pair(i, ent[e] & kIndexMask)) continue;
        const size_t sl = nl_index(v.nl_stride, i, 4 * c + e);
        if (v.S.half_stamp[sl] != stamp) continue;
        const double4_32a t = v.S.half4[sl];
        const double2 u = v.S.half2[sl];
        a.x += t.x;
        a.y += t.y;
        a.z += t.z;
        a.w += t.w;
        zw += u.x;
        sd += u.y;
      }
    }
    v.S.A4[i] = a;
    v.S.zwab[i] = zw;
    if (o.any_shepard) v.S.sumden[i] = sd;
    if (!(isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(a.w))) atomicOr(&v.sc->status, ST_NONFINITE);
    const double an = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    const double cand = o.sqrt_h_a * sqrt(Ci.h / an);
    if (cand < dtc) dtc = cand;  // NaN never compares less, as in the reference
  }
  block_dt_and_pairs<kFT>(v, Ci.inst, active, dtc, 0ull, red, cred);
}

// ---------------------------------------------------------------------------
// Soil / solid pair force (CalcForce2233) from the side of free particle i
// ---------------------------------------------------------------------------
template <int DIM, int KT>
__global__ void __launch_bounds__(kFT) forces_solid_kernel(DevView v) {
  __shared__ double red[kFT / 32];
  __shared__ unsigned long long cred[kFT / 32];
  __shared__ int qbuf[kQN][kFT];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int tid = threadIdx.x;
  const Options& o = v.o;
  const PClass* __restrict__ CT = v.cls;
  double dtc = DBL_MAX;
  unsigned long long npair2 = 0;
  bool active = false;
  int cell = -1, ci_cls = 0;
  if (i < n) {
    ci_cls = P.cls[i];
    // a domain of two materials runs this kernel for its soil or solid particles only
    const bool run = !v.inst[CT[ci_cls].inst].stop && (!o.mixed || CT[ci_cls].material != 1);
    active = run && CT[ci_cls].is_free;
    cell = v.S.cellid[i];
    if (run && !active) {
      if (!o.a_from_hook) v.S.A4[i] = make_double4_32a(o.gravity[0], o.gravity[1], o.gravity[2], 0.0);
      v.S.zwab[i] = 1.0;
      if (v.S.s_acc) v.S.s_acc[i] = 0.0;
    }
  }
  const PClass& Ci = CT[ci_cls];
  const GridDev& g = grid_of(v, Ci.inst);
  const InstState& Is = v.inst[Ci.inst];
  const bool want_s = v.S.s_acc != nullptr;
  double ss = 0.0;  // SWIType 1: the surface-erosion velocity derivative S
  const int is = active ? i : 0;
  const double4_32a xi = P.X4[is];
  const double4_32a vi = P.V4[is];
  const double4_32a di4 = v.S.D4[is];
  const double di = xi.w, inv_i = di4.x, mi = Ci.mass, hi = Ci.h;
  const bool shep = Ci.shepard && (Is.shepard_counter == o.shepard_step);
  const double* __restrict__ Si = P.sigma + 9 * (size_t)is;
  const double* __restrict__ Ti = P.tir + 9 * (size_t)is;
  double ax = o.gravity[0] + o.body_force[0], ay = o.gravity[1] + o.body_force[1],
         az = o.gravity[2] + o.body_force[2];
  double drho = 0.0, zw = 0.0, sd = 0.0, xs0 = 0.0, xs1 = 0.0, xs2 = 0.0;
  if (o.a_from_hook && active) {  // StartAcceleration's values as a GeneralBefore hook left them
    const double4_32a a0 = v.S.A4[i];
    ax = a0.x + o.body_force[0];
    ay = a0.y + o.body_force[1];
    az = a0.z + o.body_force[2];
    drho = a0.w;
  }
  double sr[6] = {0, 0, 0, 0, 0, 0}, rr[3] = {0, 0, 0};  // sr: 00 01 02 11 12 22; rr: 01 02 12
  const bool any_periodic = g.periodic[0] | g.periodic[1] | g.periodic[2];
  const double I22 = (DIM == 2) ? 0.0 : 1.0;  // Domain::I (Source/Domain.cpp:1665)
  CellCoord cci = decode(g, cell >= 0 ? cell : 0);
  NbrSource<DIM> src;
  src.init(v, g, i, active && cell >= 0, 1.004f);
  bool more = active && cell >= 0;
  while (true) {
    int qn = 0;
    while (more && qn < kQN) {
      int code;
      const int j = src.next(v, &code);
      if (j < 0) {
        more = false;
        break;
      }
      qbuf[qn++][tid] = j;
    }
    const int qmax = __reduce_max_sync(0xffffffffu, qn);
    for (int k = 0; k < qmax; ++k) {
      if (k >= qn) continue;
      const int j = qbuf[k][tid];
      const double4_32a xj = P.X4[j];
      const PClass& Cj = CT[P.cls[j]];
      if (o.mixed && Cj.material != Ci.material) continue;  // fluid partners: the coupling kernel
      const double hb = (hi + Cj.h) / 2;
      double x0 = xi.x - xj.x, x1 = xi.y - xj.y, x2 = xi.z - xj.z;
      if (any_periodic) periodic_fix(g, x0, x1, x2, hb, cci, decode(g, v.S.cellid[j]));
      const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
      const double inv_hb = o.uniform_h ? o.inv_h : 1.0 / hb;
      const double inv_r = (r2 > 0.0) ? rsqrt(r2) : 0.0;
      const double q = r2 * inv_r * inv_hb;
      if (q > g.cellfac) continue;
      const bool fj = Cj.is_free;
      npair2 += fj ? 1ull : 2ull;
      const double4_32a vj = P.V4[j];
      const bool soil = (Ci.material * Cj.material == 9);
      double dj, inv_j, cj_snd = 0.0;
      double mj;
      if (fj) {
        const double4_32a dj4 = v.S.D4[j];
        dj = xj.w; inv_j = dj4.x; cj_snd = dj4.z; mj = Cj.mass;
      } else if (soil) {  // soil walls take the partner's density (Source/Interaction.cpp:201-205)
        dj = di; inv_j = inv_i; mj = Cj.fpmassc * mi;
      } else {
        if (o.uniform_eos) {
          const double4_32a dj4 = v.S.D4[j];
          dj = dj4.w; inv_j = dj4.x; cj_snd = dj4.z;
        } else {
          dj = density_solid(Ci.pres_eq, Ci.cs, Ci.p0, vj.w, Ci.rho0);
          inv_j = 1.0 / dj;
          cj_snd = sound_speed(Ci.pres_eq, Ci.cs, dj, Ci.rho0);
        }
        mj = Cj.fpmassc * mi;
      }
      const double ih2 = inv_hb * inv_hb;
      const double cwh = Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_hb);
      const double cwg = cwh * ih2;
      const double GK = Kern<DIM, KT>::GK(q, hb * inv_r, cwg);
      const double K = Kern<DIM, KT>::W(q, cwh);
      const double v0 = vi.x - vj.x, v1 = vi.y - vj.y, v2 = vi.z - vj.z;
      const double vx = v0 * x0 + v1 * x1 + v2 * x2;
      double PIs = 0.0;  // PIij = PIs * I
      const double Alpha = (Ci.alpha + Cj.alpha) / 2.0, Beta = (Ci.beta + Cj.beta) / 2.0;
      if ((Alpha != 0.0 || Beta != 0.0) && vx < 0) {
        const double Cij = soil ? 0.5 * (Ci.cs + Cj.cs) : 0.5 * (di4.z + cj_snd);
        const double D = r2 + 0.01 * hb * hb;
        const double t = hb * vx;
        PIs = t * (Alpha * Cij * D + Beta * t) / (D * D * (0.5 * (di + dj)));
      }
      double TIs = 0.0;
      const bool ti = (Ci.ti > 0.0 || Cj.ti > 0.0);
      if (ti) {
        const double Wd = Kern<DIM, KT>::W((Ci.tid + Cj.tid) / (2.0 * hb), cwh);
        TIs = pow(K / Wd, (Ci.tin + Cj.tin) / 2.0);
      }
      double vab0, vab1, vab2;
      if (fj) { vab0 = v0; vab1 = v1; vab2 = v2; }
      else if (Ci.no_slip || Cj.no_slip) {
        const double4_32a ns = v.S.nsv4[j];
        vab0 = vi.x - (2.0 * vj.x - ns.x);
        vab1 = vi.y - (2.0 * vj.y - ns.y);
        vab2 = vi.z - (2.0 * vj.z - ns.z);
      } else {
        const double4_32a vbj = (o.scheme == PSPH_MVERLET) ? P.H4[j] : P.H4b[j];
        vab0 = vi.x - vbj.x; vab1 = vi.y - vbj.y; vab2 = vi.z - vbj.z;
      }
      const double* __restrict__ Sj = P.sigma + 9 * (size_t)j;
      const double* __restrict__ Tj = P.tir + 9 * (size_t)j;
      double M[9];
      if (o.grad_type == 0) {
        const double ci2 = inv_i * inv_i, cj2 = inv_j * inv_j;
#pragma unroll
        for (int e = 0; e < 9; ++e) M[e] = Si[e] * ci2 + Sj[e] * cj2;
      } else {
        const double c = inv_i * inv_j;
#pragma unroll
        for (int e = 0; e < 9; ++e) M[e] = (Si[e] + Sj[e]) * c;
      }
      M[0] += PIs; M[4] += PIs; M[8] += PIs * I22;
      if (ti) {
#pragma unroll
        for (int e = 0; e < 9; ++e) M[e] += (Ti[e] + Tj[e]) * TIs;
      }
      const double g0 = GK * x0, g1 = GK * x1, g2 = GK * x2;
      ax += mj * (g0 * M[0] + g1 * M[3] + g2 * M[6]);
      ay += mj * (g0 * M[1] + g1 * M[4] + g2 * M[7]);
      if (DIM == 3) az += mj * (g0 * M[2] + g1 * M[5] + g2 * M[8]);
      drho += mj * di * inv_j * (v0 * g0 + v1 * g1 + v2 * g2);
      const double md = mj * inv_j;
      zw += md * K;
      const double c2 = -0.5 * GK * md;
      sr[0] += c2 * (2.0 * vab0 * x0);
      sr[1] += c2 * (vab0 * x1 + vab1 * x0);
      sr[2] += c2 * (vab0 * x2 + vab2 * x0);
      sr[3] += c2 * (2.0 * vab1 * x1);
      sr[4] += c2 * (vab1 * x2 + vab2 * x1);
      sr[5] += c2 * (2.0 * vab2 * x2);
      rr[0] += c2 * (vab0 * x1 - vab1 * x0);
      rr[1] += c2 * (vab0 * x2 - vab2 * x0);
      rr[2] += c2 * (vab1 * x2 - vab2 * x1);
      if (o.xsph != 0.0 && fj) {
        const double s = o.xsph * mj / (0.5 * (di + dj)) * K;
        xs0 -= s * v0; xs1 -= s * v1; xs2 -= s * v2;
      }
      if (shep) sd += mj * K;
      if (want_s) ss = ss + mj / dj * vab0 * x1 * -GK;  // Source/Interaction.cpp:347
    }
    if (!__any_sync(0xffffffffu, more)) break;
  }
  if (active) {
    v.S.A4[i] = make_double4_32a(ax, ay, az, drho);
    v.S.zwab[i] = zw;
    if (o.any_shepard) v.S.sumden[i] = sd;
    if (want_s) v.S.s_acc[i] = ss;
    if (o.xsph != 0.0) v.S.vxsph4[i] = make_double4_32a(xs0, xs1, xs2, 0.0);
    double* out = v.S.strain_rate + 9 * (size_t)i;
    out[0] = sr[0]; out[1] = sr[1]; out[2] = sr[2];
    out[3] = sr[1]; out[4] = sr[3]; out[5] = sr[4];
    out[6] = sr[2]; out[7] = sr[4]; out[8] = sr[5];
    double* ro = v.S.rotation_rate + 9 * (size_t)i;
    ro[0] = 0.0; ro[1] = rr[0]; ro[2] = rr[1];
    ro[3] = -rr[0]; ro[4] = 0.0; ro[5] = rr[2];
    ro[6] = -rr[1]; ro[7] = -rr[2]; ro[8] = 0.0;
    if (!(isfinite(ax) && isfinite(ay) && isfinite(az) && isfinite(drho))) atomicOr(&v.sc->status, ST_NONFINITE);
    const double an = sqrt(ax * ax + ay * ay + az * az);
    const double cand = o.sqrt_h_a * sqrt(hi / an);
    if (cand < dtc) dtc = cand;
  }
  block_dt_and_pairs<kFT>(v, Ci.inst, active && !o.mixed, dtc, npair2, red, cred);
}

// Per-instance step control, one block looping over the instances.
// dt: LastComputeAcceleration's minimum (Source/Domain.cpp:1280-1296) and
// AdaptiveTimeStep (Source/Domain.cpp:133-152).
__global__ void dt_finalize_kernel(DevView v) {
  StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  for (int k = threadIdx.x; k < v.ninst; k += blockDim.x) {
    InstState& I = v.inst[k];
    if (I.stop) continue;
    const double m = __longlong_as_double((long long)I.dtmin_bits);
    double dtmin = I.deltatint;
    if (dtmin > m) dtmin = m;
    I.deltatmin = dtmin;
    double dt = I.deltat;
    const double dti = I.deltatint;
    if (dti > dtmin) dt = (dt < dtmin) ? 2.0 * dt * dtmin / (dt + dtmin) : dtmin;
    else dt = (dti != dt) ? 2.0 * dt * dti / (dt + dti) : dti;
    I.deltat = dt;
    if (dt < (dti / 1.0e5)) {
      atomicOr(&sc->status, ST_DT_COLLAPSE);
      I.stop = 1;  // the reference throws here (Source/Domain.cpp:150-151)
    }
  }
}

// Begin of step: Solve's `Time < tf` test per instance, Move_MVerlet's
// first-step ct (Source/Particle.cpp:191-195), reset of the dt minimum.
__global__ void begin_kernel(DevView v) {
  StepScalars* sc = v.sc;
  int live = 0;
  for (int k = threadIdx.x; k < v.ninst; k += blockDim.x) {
    InstState& I = v.inst[k];
    if (!I.stop && !(I.time < I.t_stop)) I.stop = 1;
    if (I.stop) continue;
    live = 1;
    if (v.o.scheme == PSPH_MVERLET && I.first_step) I.ct = 30;
    I.dtmin_bits = (unsigned long long)__double_as_longlong(DBL_MAX);
  }
  live = __syncthreads_or(live);
  if (threadIdx.x == 0) {
    sc->all_stop = !live;
    // the cell sort and the neighbour lists run every step, or, with a skin,
    // once a particle has moved half the skin since they last ran
    bool rb = true;
    if (v.o.skin > 0.f) rb = sc->force_rebuild || __uint_as_float(sc->disp2_bits) > v.o.skin_disp2;
    sc->rebuild = rb ? 1 : 0;
    if (rb && live) {
      sc->force_rebuild = 0;
      sc->disp2_bits = 0u;
      sc->rebuilds += 1u;
    }
  }
}

// End of step: Time += deltat and the per-particle counters, once per instance.
__global__ void end_kernel(DevView v) {
  if (v.sc->all_stop) return;
  for (int k = threadIdx.x; k < v.ninst; k += blockDim.x) {
    InstState& I = v.inst[k];
    if (I.stop) continue;
    I.time += I.deltat;
    I.steps += 1;
    if (v.o.scheme == PSPH_MVERLET) {
      I.ct = (I.ct == 30) ? 0 : I.ct + 1;
      I.shepard_counter = (I.shepard_counter == v.o.shepard_step) ? 0 : I.shepard_counter + 1;
    }
    I.first_step = 0;
    I.k_initial = 0;
  }
}

// Pair export: candidate (which=0) or in-support (which=1) pairs in reference
// orientation, as original indices; only pairs with at least one free particle
// (Source/Domain.cpp:844).
template <int DIM>
__global__ void pairs_export_kernel(DevView v, int which, long long* out, long long cap,
                                    unsigned long long* counter) {
  const int n = v.sc->n;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Persist& P = cur_persist(v);
  const int cell = v.S.cellid[i];
  if (cell < 0) return;
  const PClass* CT = v.cls;
  const PClass& Ci = CT[P.cls[i]];
  const GridDev& g = grid_of(v, Ci.inst);
  const CellCoord ci = decode(g, cell);
  const int oi = P.orig[i];
  const double4_32a xi = P.X4[i];
  for_neighbor_ranges<DIM>(g, ci, v.S.start, [&](int lo, int hi) {
    for (int j = lo; j < hi; ++j) {
      if (j == i) continue;
      const PClass& Cj = CT[P.cls[j]];
      if (!Ci.is_free && !Cj.is_free) continue;
      const CellCoord cj = decode(g, v.S.cellid[j]);
      const int oj = P.orig[j];
      if (!first_of_pair(g, ci, cj, oi, oj)) continue;  // each unordered pair once, from its first particle
      if (which == 1) {
        const double4_32a xj = P.X4[j];
        const double hb = (Ci.h + Cj.h) / 2;
        double x0 = xi.x - xj.x, x1 = xi.y - xj.y, x2 = xi.z - xj.z;
        periodic_fix(g, x0, x1, x2, hb, ci, cj);
        // the reference's expression, without contraction: sqrt(dot)/h <= Cellfac
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x0, x0), __dmul_rn(x1, x1)), __dmul_rn(x2, x2));
        if (!(__ddiv_rn(__dsqrt_rn(r2), hb) <= g.cellfac)) continue;
      }
      const unsigned long long slot = atomicAdd(counter, 1ull);
      if ((long long)slot < cap) {
        out[2 * slot] = oi;
        out[2 * slot + 1] = oj;
      }
    }
  });
}

// ---------------------------------------------------------------------------
// Fluid-soil coupling (a fluid and a soil in one domain, FP64 form)
// ---------------------------------------------------------------------------
// Saturation check (Source/Domain.cpp:1060-1089): a soil particle is saturated
// this step when a fluid particle in a neighbouring cell (a candidate pair of
// MainNeighbourSearch with one side free) lies in a cell row at or above its
// own and at or above its own height.
template <int DIM>
__global__ void __launch_bounds__(kFT) saturation_check_kernel(DevView v) {
  if (v.sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.sc->n) return;
  const PClass* __restrict__ CT = v.cls;
  const PClass& Ci = CT[P.cls[i]];
  const int cell = v.S.cellid[i];
  if (Ci.material != 3 || cell < 0 || v.inst[Ci.inst].stop) return;
  const GridDev& g = grid_of(v, Ci.inst);
  const CellCoord ci = decode(g, cell);
  const double yi = P.X4[i].y;
  bool sat = false;
  for_neighbor_ranges<DIM>(g, ci, v.S.start, [&](int lo, int hi) {
    for (int j = lo; j < hi && !sat; ++j) {
      const PClass& Cj = CT[P.cls[j]];
      if (Cj.material != 1 || !(Ci.is_free || Cj.is_free)) continue;
      if (decode(g, v.S.cellid[j]).y >= ci.y && P.X4[j].y >= yi) sat = true;
    }
  });
  v.S.satcheck[i] = sat ? 1 : 0;
}

// The weight switch that follows (Source/Domain.cpp:1209-1234): a soil particle
// whose saturation changed takes its class's twin (Mass = V (RefDensity -+ RhoF),
// RefDensity -+ RhoF) and Density, Densityb -+ RhoF; the density its partners
// see is updated with it.
__global__ void __launch_bounds__(kFT) saturation_apply_kernel(DevView v) {
  if (v.sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.sc->n) return;
  const PClass* __restrict__ CT = v.cls;
  const int q = P.cls[i];
  const PClass& C = CT[q];
  if (C.material != 3 || v.S.cellid[i] < 0 || v.inst[C.inst].stop || C.twin < 0) return;
  const bool sat = v.S.satcheck[i] != 0;
  if (sat == (C.is_sat != 0)) return;
  const double rf = C.rho_f;
  double4_32a x = P.X4[i];
  x.w = sat ? x.w - rf : x.w + rf;
  P.X4[i] = x;
  double4_32a& hb = (v.o.scheme == PSPH_MVERLET) ? P.H4[i] : P.H4b[i];  // Densityb
  double4_32a h = hb;
  h.w = sat ? h.w - rf : h.w + rf;
  hb = h;
  P.cls[i] = C.twin;
  const PClass& T = CT[C.twin];
  const double rho = x.w, inv = 1.0 / rho, pr = P.V4[i].w;
  const double snd = T.is_free ? sound_speed(T.pres_eq, T.cs, rho, T.rho0) : v.S.D4[i].z;
  v.S.D4[i] = make_double4_32a(inv, pr * inv * inv, snd, rho);
}

// Seepage (Source/Functions.cpp:266-298): Darcy (0, 1) or Forchheimer (2, 3)
PSPH_D void seepage_coeffs(int type, double k, double k2, double mu, double rho, double& sf1, double& sf2) {
  sf1 = mu / k;
  sf2 = (type >= 2) ? k2 * rho : 0.0;
}

// CalcForce13 (Source/Interaction.cpp:508-653) seen from particle i, whose
// partner j is of the other material; returns the acceleration term. Both of
// the reference's orientations give the same terms: v = v_fluid - v_soil,
// SFt = (SF1 v + SF2 |v| v) K with K = W(r/h, h) / (Density_1 Density_2) and h
// the smaller smoothing length; the soil gains m_fluid SFt (SWIType 2: minus
// m_fluid p_fluid GK x_soil,fluid), the fluid loses m_soil SFt.
template <int DIM, int KT>
PSPH_D void seepage_pair(const DevView& v, const Persist& P, const InstState& Is, int i, int j, const PClass& Ci,
                         const PClass& Cj, const double4_32a& xi, const double4_32a& xj, const double4_32a& vi,
                         double h, double x0, double x1, double x2, double r, double q, double* da) {
  const int swi = v.o.swi;
  da[0] = da[1] = da[2] = 0.0;
  if (swi == 3) return;
  const bool soil_i = (Ci.material == 3);
  const double inv_h = 1.0 / h, ih2 = inv_h * inv_h;
  const double cwh = Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_h);
  const double rr = xi.w * xj.w;
  const double K = Kern<DIM, KT>::W(q, cwh) / rr;
  // soil side s, fluid side f
  const int s = soil_i ? i : j, f = soil_i ? j : i;
  const PClass& Cs = soil_i ? Ci : Cj;
  const PClass& Cf = soil_i ? Cj : Ci;
  const double4_32a vs = soil_i ? vi : P.V4[j];
  const double4_32a vf = soil_i ? P.V4[j] : vi;
  const double w0 = vf.x - vs.x, w1 = vf.y - vs.y, w2 = vf.z - vs.z;
  const double nv = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
  double S0, S1, S2;
  bool erosion = false;
  if (swi == 1) {
    // a fixed soil particle's ZWab is 1 once CalcForce2233 saw it, else 0
    const double zw = Cs.is_free ? v.S.zwab[s] : (v.S.sumkernel[s] != 0.0 ? 1.0 : 0.0);
    erosion = zw < 0.25;
  }
  if (erosion) {  // Source/Interaction.cpp:561-566
    const double Cd = 24.0 * (Cf.mu_ref / Cf.rho0) / (Cs.dgrain * nv + 0.01 * h * h) + 2.0;
    const double c = 3.0 / (4.0 * Cs.dgrain) * Cf.rho0 * (1.0 - Cs.n0) * Cd * nv;
    S0 = c * w0 * K;
    S1 = c * w1 * K;
    S2 = c * w2 * K;
    S1 += (Cf.rho0 * (1.0 - Cs.n0) * nv * fabs(v.S.s_acc[f] - v.S.s_acc[s])) * K;
  } else {
    double kp = Cs.kp, kp2 = Cs.kp2;
    if (Cs.var_por && Cs.is_free && !Is.k_initial) {
      // VarPorosity: the permeabilities of the strain the last update left
      const double* E = P.strain + 9 * (size_t)s;
      const double ev = (E[0] + E[4] + E[8]);
      permeability(Cs.seep_type, (Cs.n0 + ev) / (1.0 + ev), Cs.dgrain, &kp, &kp2);
    }
    double sf1, sf2;
    seepage_coeffs(Cs.seep_type, kp, kp2, Cf.mu_ref, Cf.rho0, sf1, sf2);
    S0 = (sf1 * w0 + sf2 * nv * w0) * K;
    S1 = (sf1 * w1 + sf2 * nv * w1) * K;
    S2 = (sf1 * w2 + sf2 * nv * w2) * K;
  }
  if (DIM == 2) S2 = 0.0;
  if (soil_i) {
    const double mf = Cf.mass;
    da[0] = mf * S0;
    da[1] = mf * S1;
    da[2] = mf * S2;
    if (swi == 2) {  // pore pressure (Source/Interaction.cpp:608-637), x = x_soil - x_fluid
      const double GK = Kern<DIM, KT>::GK(q, h / r, cwh * ih2) / rr;
      const double c = mf * P.V4[j].w * GK;
      da[0] = da[0] - c * x0;
      da[1] = da[1] - c * x1;
      da[2] = da[2] - c * x2;
    }
  } else {
    const double ms = Cs.mass;
    da[0] = -(ms * S0);
    da[1] = -(ms * S1);
    da[2] = -(ms * S2);
  }
}

// CalcForce12 (Source/Interaction.cpp:379-507) seen from particle i, whose
// partner j is of the other material (fluid f, solid s; h the mean smoothing
// length). The solid enters with the density its FSIPressure gives under the
// fluid's EOS and the no-slip velocity 2 v_s - FSINSv; both sides take the
// fluid's mass; the reference's artificial-viscosity branch is dead (Alpha and
// Beta are zeroed before their test). The solid gains m_f temp, the fluid too
// (temp from each side's own orientation), and only the fluid gets the density
// rate and, with T0 or LES, the strain rate (added into sr).
template <int DIM, int KT>
PSPH_D void solid_pair(const DevView& v, const Persist& P, int i, int j, const PClass& Ci, const PClass& Cj,
                       const double4_32a& xi, const double4_32a& xj, const double4_32a& vi, double hb, double x0,
                       double x1, double x2, double r2, double q, double* da, double* drho, double* sr) {
  const Options& o = v.o;
  const bool fluid_i = (Ci.material == 1);
  const PClass& Cf = fluid_i ? Ci : Cj;
  const PClass& Cs = fluid_i ? Cj : Ci;
  const int s = fluid_i ? j : i, f = fluid_i ? i : j;
  const double4_32a vj = P.V4[j];
  const double rho_f = fluid_i ? xi.w : xj.w;
  const double p_f = fluid_i ? vi.w : vj.w;
  const double fp = v.S.fsi_p[s];
  const double rho_s = density_solid(Cf.pres_eq, Cf.cs, Cf.p0, fp, Cf.rho0);
  const double mf = Cf.mass;
  const double mu = o.dyn_mu ? P.mu[f] : Cf.mu0;
  const double4_32a ns = v.S.fsi_nsv[s];
  const double4_32a vs = fluid_i ? vj : vi, vf = fluid_i ? vi : vj;
  // vab from i's orientation
  const double sg = fluid_i ? 1.0 : -1.0;
  const double vab0 = sg * (vf.x - (2.0 * vs.x - ns.x)), vab1 = sg * (vf.y - (2.0 * vs.y - ns.y)),
               vab2 = sg * (vf.z - (2.0 * vs.z - ns.z));
  const double v0 = vi.x - vj.x, v1 = vi.y - vj.y, v2 = vi.z - vj.z;
  const double inv_hb = 1.0 / hb, ih2 = inv_hb * inv_hb;
  const double cwh = Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_hb);
  const double cwg = cwh * ih2;
  const double inv_r = (r2 > 0.0) ? rsqrt(r2) : 0.0;
  const double inv_q = hb * inv_r;
  const double GK = Kern<DIM, KT>::GK(q, inv_q, cwg);
  const double di = fluid_i ? rho_f : rho_s, dj = fluid_i ? rho_s : rho_f;
  double VI0, VI1, VI2;
  if (o.vis_eq <= 2) {
    double c;
    if (o.vis_eq == 0) c = 2.0 * mu / (di * dj) * GK;
    else if (o.vis_eq == 1) c = 8.0 * mu / ((di + dj) * (di + dj)) * GK;
    else c = -mu / (di * dj) * Kern<DIM, KT>::Lap(q, inv_q, cwg);
    VI0 = c * vab0; VI1 = c * vab1; VI2 = c * vab2;
  } else {
    const double L = Kern<DIM, KT>::Lap(q, inv_q, cwg);
    const double S2 = Kern<DIM, KT>::D2(q, cwg);
    const double sv = -mu / (di * dj);
    const double vx = v0 * x0 + v1 * x1 + v2 * x2;
    const double t = vx / r2 * (-GK + S2);
    VI0 = sv * (L * vab0 + (1.0 / 3.0) * (GK * v0 + t * x0));
    VI1 = sv * (L * vab1 + (1.0 / 3.0) * (GK * v1 + t * x1));
    VI2 = sv * (L * vab2 + (1.0 / 3.0) * (GK * v2 + t * x2));
  }
  double sp;
  if (o.grad_type == 0) sp = -(p_f / (rho_f * rho_f) + fp / (rho_s * rho_s)) * GK;
  else sp = -((p_f + fp) / (rho_f * rho_s)) * GK;
  da[0] = mf * (sp * x0 + VI0);
  da[1] = mf * (sp * x1 + VI1);
  da[2] = DIM == 3 ? mf * (sp * x2 + VI2) : 0.0;
  *drho = 0.0;
  if (fluid_i) {
    *drho = mf * (rho_f / rho_s) * (GK * (v0 * x0 + v1 * x1 + v2 * x2));
    if (sr && (Cf.t0 > 0.0 || Cf.les) &&
        ((Ci.t0 > 0.0 || Cj.t0 > 0.0) || (Ci.les || Cj.les))) {
      const double c2 = -GK * (mf / rho_s);
      sr[0] += c2 * (2.0 * vab0 * x0);
      sr[1] += c2 * (vab0 * x1 + vab1 * x0);
      sr[2] += c2 * (vab0 * x2 + vab2 * x0);
      sr[3] += c2 * (2.0 * vab1 * x1);
      sr[4] += c2 * (vab1 * x2 + vab2 * x1);
      sr[5] += c2 * (2.0 * vab2 * x2);
    }
  }
}

// The pairs of different materials from the side of free particle i, added in
// list order to what its own material's pair kernel wrote (CalcForce13 for
// fluid and soil, CalcForce12 for fluid and solid); then the dt bound and the
// finiteness check of the gather form.
template <int DIM, int KT>
__global__ void __launch_bounds__(kFT) coupling_kernel(DevView v) {
  __shared__ double red[kFT / 32];
  __shared__ unsigned long long cred[kFT / 32];
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const Options& o = v.o;
  const PClass* __restrict__ CT = v.cls;
  double dtc = DBL_MAX;
  unsigned long long npair2 = 0;
  bool active = false;
  int cell = -1, ci_cls = 0;
  if (i < sc->n) {
    ci_cls = P.cls[i];
    active = !v.inst[CT[ci_cls].inst].stop && CT[ci_cls].is_free;
    cell = v.S.cellid[i];
  }
  const PClass& Ci = CT[ci_cls];
  const GridDev& g = grid_of(v, Ci.inst);
  const InstState& Is = v.inst[Ci.inst];
  double4_32a a4 = active ? v.S.A4[i] : make_double4_32a(0, 0, 0, 0);
  double ax = a4.x, ay = a4.y, az = a4.z, drho = a4.w;
  if (active && cell >= 0) {
    const double4_32a xi = P.X4[i], vi = P.V4[i];
    const CellCoord cci = decode(g, cell);
    const bool any_periodic = g.periodic[0] | g.periodic[1] | g.periodic[2];
    // the fluid's strain-rate sums gain CalcForce12's terms
    const bool want_sr = o.couple_solid && o.need_sr && Ci.material == 1 && (Ci.t0 > 0.0 || Ci.les);
    double sr[6] = {0, 0, 0, 0, 0, 0};
    NbrSource<DIM> src;
    src.init(v, g, i, true, 1.004f);
    while (true) {
      int code;
      const int j = src.next(v, &code);
      if (j < 0) break;
      const PClass& Cj = CT[P.cls[j]];
      if (Cj.material == Ci.material) continue;
      // CalcForce13 takes the smaller smoothing length, CalcForce12 the mean
      const double h = o.couple_soil ? (Ci.h < Cj.h ? Ci.h : Cj.h) : (Ci.h + Cj.h) / 2;
      const double4_32a xj = P.X4[j];
      double x0 = xi.x - xj.x, x1 = xi.y - xj.y, x2 = xi.z - xj.z;
      if (any_periodic) periodic_fix(g, x0, x1, x2, h, cci, decode(g, v.S.cellid[j]));
      const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
      const double r = sqrt(r2);
      const double q = r / h;
      if (!(q <= g.cellfac)) continue;
      npair2 += Cj.is_free ? 1ull : 2ull;
      double da[3], dr = 0.0;
      if (o.couple_soil) {
        seepage_pair<DIM, KT>(v, P, Is, i, j, Ci, Cj, xi, xj, vi, h, x0, x1, x2, r, q, da);
      } else {
        solid_pair<DIM, KT>(v, P, i, j, Ci, Cj, xi, xj, vi, h, x0, x1, x2, r2, q, da, &dr, want_sr ? sr : nullptr);
      }
      ax += da[0];
      ay += da[1];
      az += da[2];
      drho += dr;
    }
    v.S.A4[i] = make_double4_32a(ax, ay, az, drho);
    if (want_sr) {
      double* out = v.S.strain_rate + 9 * (size_t)i;
      out[0] += sr[0]; out[1] += sr[1]; out[2] += sr[2];
      out[3] += sr[1]; out[4] += sr[3]; out[5] += sr[4];
      out[6] += sr[2]; out[7] += sr[4]; out[8] += sr[5];
    }
    if (!(isfinite(ax) && isfinite(ay) && isfinite(az) && isfinite(drho))) atomicOr(&v.sc->status, ST_NONFINITE);
    const double an = sqrt(ax * ax + ay * ay + az * az);
    const double cand = o.sqrt_h_a * sqrt(Ci.h / an);
    if (cand < dtc) dtc = cand;
  } else if (active) {
    const double an = sqrt(ax * ax + ay * ay + az * az);
    const double cand = o.sqrt_h_a * sqrt(Ci.h / an);
    if (cand < dtc) dtc = cand;
  }
  block_dt_and_pairs<kFT>(v, Ci.inst, active, dtc, npair2, red, cred);
}

// FSI interpolation (Source/Domain.cpp:1090-1160): a free solid particle takes
// FSIPressure = sum(p_f K + (g.x) rho_f K) and FSINSv = sum(v_f K) over its free
// fluid candidates (K = 0 outside the support), divided by the kernel sum once
// per candidate, as the reference's normalisation loop runs once per entry of
// FreeFSIParticles (one entry per pair; with Nproc = 1). As in the reference,
// the gravity term's x is x_first - x_second of MainNeighbourSearch's pair, and
// only pairs that list the solid first add to FSINSv (the others add to the
// solid's NSv, which nothing reads for a free particle). Fixed solids get 0.
template <int DIM, int KT>
__global__ void __launch_bounds__(kFT) fsi_kernel(DevView v) {
  if (v.sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.sc->n) return;
  const PClass* __restrict__ CT = v.cls;
  const PClass& Ci = CT[P.cls[i]];
  const int cell = v.S.cellid[i];
  if (Ci.material != 2 || v.inst[Ci.inst].stop) return;
  double sk = 0.0, sp = 0.0, n0 = 0.0, n1 = 0.0, n2 = 0.0;
  int cnt = 0;
  if (Ci.is_free && cell >= 0) {
    const GridDev& g = grid_of(v, Ci.inst);
    const CellCoord ci = decode(g, cell);
    const double4_32a xi = P.X4[i];
    const int oi = P.orig[i];
    const double gx = v.o.gravity[0], gy = v.o.gravity[1], gz = v.o.gravity[2];
    const bool any_periodic = g.periodic[0] | g.periodic[1] | g.periodic[2];
    for_neighbor_ranges<DIM>(g, ci, v.S.start, [&](int lo, int hi) {
      for (int j = lo; j < hi; ++j) {
        const PClass& Cj = CT[P.cls[j]];
        if (Cj.material != 1 || !Cj.is_free) continue;
        const CellCoord cj = decode(g, v.S.cellid[j]);
        const bool solid_first = first_of_pair(g, ci, cj, oi, P.orig[j]);
        const double4_32a xj = P.X4[j], vj = P.V4[j];
        const double hb = (Ci.h + Cj.h) / 2.0;
        double x0, x1, x2;
        if (solid_first) {
          x0 = xi.x - xj.x; x1 = xi.y - xj.y; x2 = xi.z - xj.z;
          if (any_periodic) periodic_fix(g, x0, x1, x2, hb, ci, cj);
        } else {
          x0 = xj.x - xi.x; x1 = xj.y - xi.y; x2 = xj.z - xi.z;
          if (any_periodic) periodic_fix(g, x0, x1, x2, hb, cj, ci);
        }
        const double inv_hb = 1.0 / hb, ih2 = inv_hb * inv_hb;
        const double K = Kern<DIM, KT>::W(sqrt(x0 * x0 + x1 * x1 + x2 * x2) * inv_hb,
                                          Kern<DIM, KT>::cw() * (DIM == 2 ? ih2 : ih2 * inv_hb));
        ++cnt;
        sk += K;
        if (solid_first) { n0 += vj.x * K; n1 += vj.y * K; n2 += vj.z * K; }
        sp += vj.w * K + (gx * x0 + gy * x1 + gz * x2) * xj.w * K;
      }
    });
    for (int c = 0; c < cnt; ++c) {
      sp = sp / sk;
      n0 = n0 / sk; n1 = n1 / sk; n2 = n2 / sk;
    }
  }
  v.S.fsi_p[i] = sp;
  v.S.fsi_nsv[i] = make_double4_32a(n0, n1, n2, 0.0);
}

inline int nblk(int n, int bt) { return n <= 0 ? 1 : (n + bt - 1) / bt; }

template <int DIM>
void prepare_dispatch(const DevView& v, cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  switch (v.o.kt) {
    case 0: prepare_wall_kernel<DIM, 0><<<nb, kFT, 0, st>>>(v); break;
    case 1: prepare_wall_kernel<DIM, 1><<<nb, kFT, 0, st>>>(v); break;
    default: prepare_wall_kernel<DIM, 2><<<nb, kFT, 0, st>>>(v); break;
  }
}

template <int DIM>
void forces_dispatch(const DevView& v, cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.has_solid) {
    if (v.o.mixed) {  // fluid-soil: the fluid's pairs, then the soil's (each kernel keeps to its material)
      switch (v.o.kt) {
        case 0: forces_fluid_kernel<DIM, 0, false><<<nb, kFT, 0, st>>>(v); break;
        case 1: forces_fluid_kernel<DIM, 1, false><<<nb, kFT, 0, st>>>(v); break;
        default: forces_fluid_kernel<DIM, 2, false><<<nb, kFT, 0, st>>>(v); break;
      }
    }
    switch (v.o.kt) {
      case 0: forces_solid_kernel<DIM, 0><<<nb, kFT, 0, st>>>(v); break;
      case 1: forces_solid_kernel<DIM, 1><<<nb, kFT, 0, st>>>(v); break;
      default: forces_solid_kernel<DIM, 2><<<nb, kFT, 0, st>>>(v); break;
    }
  } else if (v.o.fp64_half) {  // each pair once: pass A, then the partners' terms
    switch (v.o.kt) {
      case 0:
        forces_fluid_kernel<DIM, 0, true><<<nb, kFT, 0, st>>>(v);
        forces_fluid_fold_kernel<DIM><<<nb, kFT, 0, st>>>(v);
        break;
      case 1:
        forces_fluid_kernel<DIM, 1, true><<<nb, kFT, 0, st>>>(v);
        forces_fluid_fold_kernel<DIM><<<nb, kFT, 0, st>>>(v);
        break;
      default:
        forces_fluid_kernel<DIM, 2, true><<<nb, kFT, 0, st>>>(v);
        forces_fluid_fold_kernel<DIM><<<nb, kFT, 0, st>>>(v);
        break;
    }
  } else {
    switch (v.o.kt) {
      case 0: forces_fluid_kernel<DIM, 0, false><<<nb, kFT, 0, st>>>(v); break;
      case 1: forces_fluid_kernel<DIM, 1, false><<<nb, kFT, 0, st>>>(v); break;
      default: forces_fluid_kernel<DIM, 2, false><<<nb, kFT, 0, st>>>(v); break;
    }
  }
}

}  // namespace

int forces_blocks(int ncap) { return nblk(ncap, kFT); }

void launch_prepare(const DevView& v, cudaStream_t st) {
  if (v.o.dim == 2) prepare_dispatch<2>(v, st);
  else prepare_dispatch<3>(v, st);
}

void launch_wall(const DevView&, cudaStream_t) {}  // fused into launch_prepare

void launch_forces(const DevView& v, cudaStream_t st) {
  if (v.o.dim == 2) forces_dispatch<2>(v, st);
  else forces_dispatch<3>(v, st);
}

void launch_saturation(const DevView& v, cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.dim == 2) saturation_check_kernel<2><<<nb, kFT, 0, st>>>(v);
  else saturation_check_kernel<3><<<nb, kFT, 0, st>>>(v);
  saturation_apply_kernel<<<nb, kFT, 0, st>>>(v);
}

template <template <int, int> class Launch>
void by_dim_kernel(const DevView& v, cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.dim == 2) {
    switch (v.o.kt) {
      case 0: Launch<2, 0>::run(v, nb, st); break;
      case 1: Launch<2, 1>::run(v, nb, st); break;
      default: Launch<2, 2>::run(v, nb, st); break;
    }
  } else {
    switch (v.o.kt) {
      case 0: Launch<3, 0>::run(v, nb, st); break;
      case 1: Launch<3, 1>::run(v, nb, st); break;
      default: Launch<3, 2>::run(v, nb, st); break;
    }
  }
}
template <int DIM, int KT>
struct CouplingLaunch {
  static void run(const DevView& v, int nb, cudaStream_t st) { coupling_kernel<DIM, KT><<<nb, kFT, 0, st>>>(v); }
};
template <int DIM, int KT>
struct FsiLaunch {
  static void run(const DevView& v, int nb, cudaStream_t st) { fsi_kernel<DIM, KT><<<nb, kFT, 0, st>>>(v); }
};

void launch_coupling(const DevView& v, cudaStream_t st) { by_dim_kernel<CouplingLaunch>(v, st); }

void launch_fsi(const DevView& v, cudaStream_t st) { by_dim_kernel<FsiLaunch>(v, st); }

void launch_dt(const DevView& v, cudaStream_t st) { dt_finalize_kernel<<<1, 256, 0, st>>>(v); }

void launch_begin(const DevView& v, cudaStream_t st) { begin_kernel<<<1, 256, 0, st>>>(v); }

void launch_end(const DevView& v, cudaStream_t st) { end_kernel<<<1, 256, 0, st>>>(v); }

void launch_pairs_export(const DevView& v, int which, long long* out, long long cap, unsigned long long* counter,
                         cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.dim == 2) pairs_export_kernel<2><<<nb, kFT, 0, st>>>(v, which, out, cap, counter);
  else pairs_export_kernel<3><<<nb, kFT, 0, st>>>(v, which, out, cap, counter);
}

}  // namespace psph

// ---------------------------------------------------------------------------
// Two-pass pair export (count, then write at scanned offsets): the same pairs
// as pairs_export_kernel, in sorted-particle order, with no atomic counter.
// Its scratch (per-particle counts and offsets) is supplied by the caller.
// ---------------------------------------------------------------------------
namespace psph {
namespace {

template <int DIM>
PSPH_D int pairs_of_particle(const DevView& v, int i, int which, long long* out, long long base, long long cap) {
  const Persist& P = cur_persist(v);
  const int cell = v.S.cellid[i];
  if (cell < 0) return 0;
  const PClass* CT = v.cls;
  const PClass& Ci = CT[P.cls[i]];
  const GridDev& g = grid_of(v, Ci.inst);
  const CellCoord ci = decode(g, cell);
  const int oi = P.orig[i];
  const double4_32a xi = P.X4[i];
  int k = 0;
  for_neighbor_ranges<DIM>(g, ci, v.S.start, [&](int lo, int hi) {
    for (int j = lo; j < hi; ++j) {
      if (j == i) continue;
      const PClass& Cj = CT[P.cls[j]];
      if (!Ci.is_free && !Cj.is_free) continue;
      const CellCoord cj = decode(g, v.S.cellid[j]);
      const int oj = P.orig[j];
      if (!first_of_pair(g, ci, cj, oi, oj)) continue;
      if (which == 1) {
        const double4_32a xj = P.X4[j];
        const double hb = (Ci.h + Cj.h) / 2;
        double x0 = xi.x - xj.x, x1 = xi.y - xj.y, x2 = xi.z - xj.z;
        periodic_fix(g, x0, x1, x2, hb, ci, cj);
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(x0, x0), __dmul_rn(x1, x1)), __dmul_rn(x2, x2));
        if (!(__ddiv_rn(__dsqrt_rn(r2), hb) <= g.cellfac)) continue;
      }
      if (out) {
        const long long slot = base + k;
        if (slot < cap) {
          out[2 * slot] = oi;
          out[2 * slot + 1] = oj;
        }
      }
      ++k;
    }
  });
  return k;
}

template <int DIM>
__global__ void pairs_count_kernel(DevView v, int which, int* __restrict__ counts, int ncap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncap) return;
  counts[i] = (i < v.sc->n) ? pairs_of_particle<DIM>(v, i, which, nullptr, 0, 0) : 0;
}

template <int DIM>
__global__ void pairs_write_kernel(DevView v, int which, const int* __restrict__ offsets, long long* out,
                                   long long cap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.sc->n) return;
  pairs_of_particle<DIM>(v, i, which, out, offsets[i], cap);
}

}  // namespace

void launch_pairs_count(const DevView& v, int which, int* counts, cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.dim == 2) pairs_count_kernel<2><<<nb, kFT, 0, st>>>(v, which, counts, v.ncap);
  else pairs_count_kernel<3><<<nb, kFT, 0, st>>>(v, which, counts, v.ncap);
}

void launch_pairs_write(const DevView& v, int which, const int* offsets, long long* out, long long cap,
                        cudaStream_t st) {
  const int nb = nblk(v.ncap, kFT);
  if (v.o.dim == 2) pairs_write_kernel<2><<<nb, kFT, 0, st>>>(v, which, offsets, out, cap);
  else pairs_write_kernel<3><<<nb, kFT, 0, st>>>(v, which, offsets, out, cap);
}

}  // namespace psph
