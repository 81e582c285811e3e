// Fused per-particle update: Domain::Move (Source/Domain.cpp:1299-1325) ->
// Particle::Move (Source/Particle.cpp:119-144) with Move_Leapfrog (:561-596)
// or Move_MVerlet (:189-274), the material update Mat1 (:146-186), Mat2*
// (:276-318, :598-639) or Mat3* (:320-482, :641-795), the periodic wrap, and
// CheckParticleLeave's test (Source/Domain.cpp:517-547; removal happens in the
// next cell sort). One thread per particle, state read and written once.
#include "psph_device.cuh"

namespace psph {

namespace {

constexpr int kUT = 128;

PSPH_D void mat_mult(const double* A, const double* B, double* M) {  // External/matvec.h:814-820
  M[0] = A[2] * B[6] + A[1] * B[3] + A[0] * B[0];
  M[1] = A[2] * B[7] + A[1] * B[4] + A[0] * B[1];
  M[2] = A[2] * B[8] + A[1] * B[5] + A[0] * B[2];
  M[3] = A[5] * B[6] + B[3] * A[4] + B[0] * A[3];
  M[4] = A[5] * B[7] + A[4] * B[4] + B[1] * A[3];
  M[5] = A[5] * B[8] + A[4] * B[5] + B[2] * A[3];
  M[6] = A[8] * B[6] + B[3] * A[7] + B[0] * A[6];
  M[7] = B[7] * A[8] + B[4] * A[7] + B[1] * A[6];
  M[8] = A[8] * B[8] + B[5] * A[7] + B[2] * A[6];
}

PSPH_D double J2of(const double* S) {
  return 0.5 * (S[0] * S[0] + 2.0 * S[1] * S[3] + 2.0 * S[2] * S[6] + S[4] * S[4] + 2.0 * S[5] * S[7] + S[8] * S[8]);
}

// Plane strain (2D): a tensor's xz, yz, zx and zy entries (2, 5, 6, 7) are
// exact zeros in the strain rate, the stresses and the strains, and the
// rotation rate holds only its xy / yx entries, when particles share one z and
// v_z = 0 (the update zeroes it). Every product with those entries is then an
// exact zero, so PL = true evaluates the same expressions on entries 0, 1, 3,
// 4, 8 only and stores zeros in the rest (the FP64 pipe bounds this kernel).
// live<PL>(e): entry e is evaluated.
template <bool PL>
PSPH_D constexpr bool live(int e) {
  return !PL || (e != 2 && e != 5 && e != 6 && e != 7);
}

template <bool PL>
PSPH_D double J2of_t(const double* S) {
  if (!PL) return J2of(S);
  return 0.5 * (S[0] * S[0] + 2.0 * S[1] * S[3] + S[4] * S[4] + S[8] * S[8]);
}

// True when the entries that PL = true leaves out are zeros (either sign) in
// every tensor the Mat3 update and the strain integration read.
PSPH_D bool plane_zeros(const double* SR, const double* RR, const double* Sig, const double* Sh, const double* E,
                        const double* Eh) {
  unsigned long long b = 0;
  const double* T[6] = {SR, RR, Sig, Sh, E, Eh};
#pragma unroll
  for (int t = 0; t < 6; ++t)
    b |= (unsigned long long)__double_as_longlong(T[t][2]) | (unsigned long long)__double_as_longlong(T[t][5]) |
         (unsigned long long)__double_as_longlong(T[t][6]) | (unsigned long long)__double_as_longlong(T[t][7]);
  b |= (unsigned long long)__double_as_longlong(RR[0]) | (unsigned long long)__double_as_longlong(RR[4]) |
       (unsigned long long)__double_as_longlong(RR[8]);
  return (b << 1) == 0ull;
}

PSPH_D double OIe(int e) { return (e == 0 || e == 4 || e == 8) ? 1.0 : 0.0; }

// 2G(D - tr D/3 I) + S W^T + W S (solid, around ShearStress)
PSPH_D void mat2_rate(const double* SR, const double* RR, const double* SS, double G, double* X) {
  double RRT[9], SRT[9], RS[9];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) RRT[3 * r + c] = RR[3 * c + r];
  mat_mult(SS, RRT, SRT);
  mat_mult(RR, SS, RS);
  const double s_tr = 1.0 / 3.0 * (SR[0] + SR[4] + SR[8]);
  const double g2 = 2.0 * G;
  for (int e = 0; e < 9; ++e) X[e] = (((SR[e] - OIe(e) * s_tr) * g2) + SRT[e]) + RS[e];
}

// K tr(D) I + 2G(D - tr D/3 I) + Sigma W^T + W Sigma (soil, around Sigma)
template <bool PL>
PSPH_D void mat3_rate(const double* SR, const double* RR, const double* Sg, double K, double G, double* X) {
  double SRT[9], RS[9];
  if (PL) {  // W = RR[1] (xy), RR[3] (yx): the nonzero terms of mat_mult's sums
    SRT[0] = Sg[1] * RR[1]; SRT[1] = Sg[0] * RR[3]; SRT[3] = Sg[4] * RR[1]; SRT[4] = Sg[3] * RR[3];
    RS[0] = RR[1] * Sg[3]; RS[1] = RR[1] * Sg[4]; RS[3] = RR[3] * Sg[0]; RS[4] = RR[3] * Sg[1];
    SRT[8] = RS[8] = 0.0;
  } else {
    double RRT[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) RRT[3 * r + c] = RR[3 * c + r];
    mat_mult(Sg, RRT, SRT);
    mat_mult(RR, Sg, RS);
  }
  const double I1s = SR[0] + SR[4] + SR[8];
  const double sK = I1s * K, s3 = 1.0 / 3.0 * I1s, g2 = 2.0 * G;
#pragma unroll
  for (int e = 0; e < 9; ++e) {
    if (!live<PL>(e)) { X[e] = 0.0; continue; }
    if (PL && e == 8) X[e] = sK + ((SR[e] - s3) * g2);
    else X[e] = ((OIe(e) * sK + ((SR[e] - OIe(e) * s3) * g2)) + SRT[e]) + RS[e];
  }
}

PSPH_D double dp_apex(double* S, double alpha, double kf) {
  double I1 = S[0] + S[4] + S[8];
  if ((kf - alpha * I1) < 0.0) {
    const double Ratio = (alpha == 0.0) ? 0.0 : kf / alpha;
    S[0] -= 1.0 / 3.0 * (I1 - Ratio);
    S[4] -= 1.0 / 3.0 * (I1 - Ratio);
    S[8] -= 1.0 / 3.0 * (I1 - Ratio);
    I1 = Ratio;
  }
  return I1;
}

template <bool PL = false>
PSPH_D void deviator(const double* S, double I1, double* D) {
  const double s = 1.0 / 3.0 * I1;
#pragma unroll
  for (int e = 0; e < 9; ++e) D[e] = live<PL>(e) ? S[e] - OIe(e) * s : 0.0;
}

// Drucker-Prager return (Source/Particle.cpp:357-425 / :677-746).
// Sig: elastic predictor (in/out); Sn: stress at the start of the step;
// fac: dt (leapfrog / restart) or 2 dt (Verlet). Returns the last deviator.
// Drucker-Prager alpha and k_f: plane strain when I(2,2) == 0 (2D), else
// the compression-cone fit (Source/Particle.cpp:663-674).
PSPH_D void dp_constants(double phi, double c, double I22, double* alpha, double* kf) {
  if (I22 == 0.0) {
    *alpha = tan(phi) / sqrt(9.0 + 12.0 * tan(phi) * tan(phi));
    *kf = 3.0 * c / sqrt(9.0 + 12.0 * tan(phi) * tan(phi));
  } else {
    *alpha = (2.0 * sin(phi)) / (sqrt(3.0) * (3.0 - sin(phi)));
    *kf = (6.0 * c * cos(phi)) / (sqrt(3.0) * (3.0 - sin(phi)));
  }
}

template <bool PL>
PSPH_D void dp_return(const PClass& C, double I22, double* Sig, const double* Sn, const double* SR, double I1strain,
                      double fac, double* SS) {
  const double alpha = C.dp_alpha, kf = C.dp_kf;  // dp_constants of the class (class_constants_kernel)
  const double K = C.k_mod, G = C.g_mod;
  double I1 = dp_apex(Sig, alpha, kf);
  deviator<PL>(Sig, I1, SS);
  double J2 = J2of_t<PL>(SS);
  if ((sqrt(J2) + alpha * I1 - kf) > 0.0) {
    deviator<PL>(Sn, Sn[0] + Sn[4] + Sn[8], SS);
    J2 = J2of_t<PL>(SS);
    if (sqrt(J2) > 0.0) {
      double sum = SS[0] * SR[0];
#pragma unroll
      for (int e = 1; e < 9; ++e)
        if (live<PL>(e)) sum = sum + SS[e] * SR[e];
      const double gj = G / sqrt(J2);
      double dL, s;
      if (C.fail == 2) {
        dL = 1.0 / (9.0 * alpha * alpha * K + G) * ((3.0 * alpha * K * I1strain) + (G / sqrt(J2)) * sum);
        s = 3.0 * alpha * K;
      } else {
        dL = 1.0 / (9.0 * alpha * K * 3.0 * C.dp_sin_psi + G) * ((3.0 * alpha * K * I1strain) + (G / sqrt(J2)) * sum);
        s = 3.0 * 3.0 * C.dp_sin_psi * K;
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) {
        if (!live<PL>(e)) continue;  // stays zero
        const double Ie = (e == 8) ? I22 : OIe(e);
        Sig[e] = Sig[e] - ((Ie * s + SS[e] * gj) * dL) * fac;
      }
    }
    I1 = dp_apex(Sig, alpha, kf);
    deviator<PL>(Sig, I1, SS);
    J2 = J2of_t<PL>(SS);
    if ((sqrt(J2) + alpha * I1 - kf) > 0.0 && sqrt(J2) > 0.0) {
      const double s1 = I1 / 3.0, s2 = (kf - alpha * I1) / sqrt(J2);
#pragma unroll
      for (int e = 0; e < 9; ++e)
        if (live<PL>(e)) Sig[e] = OIe(e) * s1 + SS[e] * s2;
    }
  }
}

// Mat3Leapfrog / Mat3MVerlet (Source/Particle.cpp:641-795 / :320-482) on one
// particle's stress: Sig (in/out), Sh (the half-step or previous stress),
// So (scratch), SS (the deviator out, when the state keeps one).
template <bool PL>
PSPH_D void mat3_update(const PClass& C, double I22, bool lf, int first, int ct, double dt, const double* SR,
                        const double* RR, double* Sig, double* Sh, double* So, double* SS) {
  double X9[9], Sn[9], SSd[9];
  mat3_rate<PL>(SR, RR, Sig, C.k_mod, C.g_mod, X9);
  const double I1strain = SR[0] + SR[4] + SR[8];
#pragma unroll
  for (int e = 0; e < 9; ++e) Sn[e] = live<PL>(e) ? Sig[e] : 0.0;
  bool have_dev = false;
  if (lf) {
    if (first)
#pragma unroll
      for (int e = 0; e < 9; ++e) Sh[e] = live<PL>(e) ? X9[e] * (-dt / 2.0) + Sig[e] : 0.0;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      if (!live<PL>(e)) { So[e] = Sh[e] = 0.0; continue; }
      So[e] = Sh[e];
      Sh[e] = X9[e] * dt + Sh[e];
    }
    if (C.fail > 1) { dp_return<PL>(C, I22, Sh, Sn, SR, I1strain, dt, SSd); have_dev = true; }
#pragma unroll
    for (int e = 0; e < 9; ++e) Sig[e] = live<PL>(e) ? (Sh[e] + So[e]) * (1.0 / 2.0) : 0.0;
  } else {
#pragma unroll
    for (int e = 0; e < 9; ++e)
      Sig[e] = !live<PL>(e) ? 0.0 : (ct == 30) ? X9[e] * dt + Sig[e] : X9[e] * (2.0 * dt) + Sh[e];
#pragma unroll
    for (int e = 0; e < 9; ++e) Sh[e] = Sn[e];
    if (C.fail > 1) { dp_return<PL>(C, I22, Sig, Sn, SR, I1strain, (ct == 30) ? dt : 2.0 * dt, SSd); have_dev = true; }
  }
  if (have_dev && SS)
#pragma unroll
    for (int e = 0; e < 9; ++e) SS[e] = SSd[e];
}

// Strain integration of Mat2 and Mat3 (the same Leapfrog / MVerlet steps as
// the stress).
template <bool PL>
PSPH_D void strain_update(bool lf, int first, int ct, double dt, const double* SR, double* E, double* Eh, double* Eo) {
  if (lf) {
    if (first)
#pragma unroll
      for (int e = 0; e < 9; ++e) Eh[e] = live<PL>(e) ? SR[e] * (-dt / 2.0) + E[e] : 0.0;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      if (!live<PL>(e)) { Eo[e] = Eh[e] = E[e] = 0.0; continue; }
      Eo[e] = Eh[e];
      Eh[e] = SR[e] * dt + Eh[e];
      E[e] = (Eh[e] + Eo[e]) * (1.0 / 2.0);
    }
  } else {
#pragma unroll
    for (int e = 0; e < 9; ++e) {
      if (!live<PL>(e)) { E[e] = Eh[e] = 0.0; continue; }
      const double old = E[e];
      E[e] = (ct == 30) ? SR[e] * dt + E[e] : SR[e] * (2.0 * dt) + Eh[e];
      Eh[e] = old;
    }
  }
}

template <int DIM>
__global__ void __launch_bounds__(kUT) update_kernel(DevView v) {
  const StepScalars* sc = v.sc;
  if (sc->all_stop) return;
  const Persist& P = cur_persist(v);
  const int n = sc->n;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const PClass& C = v.cls[P.cls[s]];
  if (!C.is_free) return;
  const InstState& Is = v.inst[C.inst];
  if (Is.stop) return;
  const Options& o = v.o;
  const GridDev& g = grid_of(v, C.inst);
  const double dt = Is.deltat;
  const int first = Is.first_step;
  const int ct = Is.ct;
  double4_32a X = P.X4[s];
  double4_32a V = P.V4[s];
  double4_32a H = P.H4[s];
  double4_32a A = v.S.A4[s];
  if (P.io && P.io[s] > 0) {
    // in/out-flow particles keep their prescribed state (Source/Domain.cpp:1305-1320)
    A.x = A.y = A.z = 0.0;
    if (P.io[s] == 1 || o.out_density > 0.0) {
      A.w = 0.0;
      v.S.zwab[s] = 0.0;
    }
    v.S.A4[s] = A;
  }
  double x[3] = {X.x, X.y, X.z}, vel[3] = {V.x, V.y, V.z};
  const double a[3] = {A.x, A.y, A.z};
  const double drho = A.w;
  double rho = X.w;
  if (o.scheme == PSPH_MVERLET) {
    // Move_MVerlet (Source/Particle.cpp:189-274)
    double vx[3] = {0.0, 0.0, 0.0};
    if (o.xsph != 0.0) {
      const double4_32a w = v.S.vxsph4[s];
      vx[0] = w.x; vx[1] = w.y; vx[2] = w.z;
    }
    for (int d = 0; d < 3; ++d) x[d] += dt * (vel[d] + vx[d]) + 0.5 * dt * dt * a[d];
    const bool shep = C.shepard && (Is.shepard_counter == o.shepard_step);
    const double zw = v.S.zwab[s];
    double rhob = H.w;
    double vb[3] = {H.x, H.y, H.z};
    if (ct == 30) {
      if (shep && zw > 0.6) {
        const double sd = v.S.sumden[s];
        rhob = sd / zw;
        rho = sd / zw;
      } else {
        rhob = rho;
        rho += dt * drho;
      }
      for (int d = 0; d < 3; ++d) {
        vb[d] = vel[d];
        vel[d] += dt * a[d];
      }
    } else {
      if (shep && zw > 0.6) {
        const double sd = v.S.sumden[s];
        rhob = sd / zw;
        rho = sd / zw;
      } else {
        const double dens = rho;
        rho = rhob + 2.0 * dt * drho;
        rhob = dens;
      }
      for (int d = 0; d < 3; ++d) {
        const double t = vel[d];
        vel[d] = vb[d] + 2 * dt * a[d];
        vb[d] = t;
      }
    }
    H = make_double4_32a(vb[0], vb[1], vb[2], rhob);
  } else {
    // Move_Leapfrog (Source/Particle.cpp:561-596)
    double va[3] = {H.x, H.y, H.z};
    double rhoa = H.w;
    if (first) {
      rhoa = rho - dt / 2.0 * drho;
      for (int d = 0; d < 3; ++d) va[d] = vel[d] - dt / 2.0 * a[d];
    }
    const double rhob = rhoa;
    rhoa += dt * drho;
    rho = (rhoa + rhob) / 2.0;
    double vb[3];
    for (int d = 0; d < 3; ++d) {
      vb[d] = va[d];
      va[d] += dt * a[d];
      vel[d] = (va[d] + vb[d]) / 2.0;
      x[d] += dt * va[d];
    }
    H = make_double4_32a(va[0], va[1], va[2], rhoa);
    P.H4b[s] = make_double4_32a(vb[0], vb[1], vb[2], rhob);
  }
  double p = V.w;
  const int mat = C.material;
  if (mat == 1) {
    // Mat1 (Source/Particle.cpp:146-186)
    if (o.fp32 && C.pres_eq == 1) {
      // FP32C: the Tait pressure from d = rho/rho0 - 1 (FP64) as p0 + B ((1+d)^7 - 1)
      // with the power expanded, 7d + 21d^2 + ... + d^7, in FP32: no cancellation
      // near rho0, ~1e-7 relative, 5 FP64 operations instead of two divisions
      const float e = (float)((rho - C.rho0) * C.eos_inv_rho0);
      const float poly = e * (7.f + e * (21.f + e * (35.f + e * (35.f + e * (21.f + e * (7.f + e))))));
      p = C.p0 + (double)(C.eos_b32 * poly);
    } else {
      p = eos(C.pres_eq, C.cs, C.p0, rho, C.rho0);
    }
    if (o.need_sr || o.dyn_mu) {
      double shear_rate = 0.0, sbar = 0.0;
      if (o.need_sr && o.fp32 && !o.has_solid) {
        // FP32C fluid pair kernel: its FP32 contraction of its FP32 sums (two
        // FP64 square roots per particle less); Sbar = sqrt(2 temp) = 2 ShearRate
        shear_rate = (double)v.S.cshear[s];
        sbar = 2.0 * shear_rate;
      } else if (o.need_sr) {
        const double* S = v.S.strain_rate + 9 * (size_t)s;
        const double temp =
            (S[0] * S[0] + 2.0 * S[1] * S[3] + 2.0 * S[2] * S[6] + S[4] * S[4] + 2.0 * S[5] * S[7] + S[8] * S[8]);
        shear_rate = sqrt(0.5 * temp);
        sbar = sqrt(2.0 * temp);
      }
      v.S.shear_rate[s] = shear_rate;
      v.S.sbar[s] = sbar;
      if (o.dyn_mu) {
        double mu = P.mu[s];
        if (C.les) {
          const double nut = o.closure ? v.S.nut[s] : -1.0;
          if (nut >= 0.0) {
            mu = C.mu_ref + C.rho0 * nut;  // learned eddy viscosity
          } else {
            const double ch = C.csmag * C.h;
            mu = C.mu_ref + C.rho0 * (ch * ch) * sbar;
          }
        }
        if (C.t0 > 0.0) {
          // Bingham (Source/Particle.cpp:166-170): 1-exp(-m g) evaluated as -expm1(-m g),
          // the same function without the cancellation that makes the reference's
          // form return T0*0 instead of T0*m for shear rates below ~1e-16/m
          if (C.vis_m == 0) mu = (shear_rate != 0.0) ? C.mu_ref + C.t0 * (-expm1(-C.bm * shear_rate)) / shear_rate
                                                    : C.mu_ref + C.t0 * C.bm;
          else mu = (1000.0 * C.mu_ref + C.mu_ref * C.mu_ref * 1000.0 / C.t0 * shear_rate) /
                    (1 + 1000.0 * C.mu_ref / C.t0 * shear_rate);
        }
        P.mu[s] = mu;
      }
    }
  } else {
    const double* SR = v.S.strain_rate + 9 * (size_t)s;
    const double* RR = v.S.rotation_rate + 9 * (size_t)s;
    double* Sig = P.sigma + 9 * (size_t)s;
    double* Sh = P.sigma_h + 9 * (size_t)s;
    double* So = v.S.sigma_o + 9 * (size_t)s;
    double* E = P.strain + 9 * (size_t)s;
    double* Eh = P.strain_h + 9 * (size_t)s;
    double* Eo = v.S.strain_o + 9 * (size_t)s;
    const double I22 = (DIM == 2) ? 0.0 : 1.0;
    const bool lf = (o.scheme != PSPH_MVERLET);
    bool plane = false;
    if (mat == 2) {
      // Mat2Leapfrog / Mat2MVerlet (Source/Particle.cpp:598-639 / :276-318)
      p = eos(C.pres_eq, C.cs, C.p0, rho, C.rho0);
      double* SS = P.shear + 9 * (size_t)s;
      double* SSh = P.shear_h + 9 * (size_t)s;
      double* SSo = v.S.shear_o + 9 * (size_t)s;
      double X9[9];
      mat2_rate(SR, RR, SS, C.g_mod, X9);
      double* target;
      if (lf) {
        if (first)
          for (int e = 0; e < 9; ++e) SSh[e] = X9[e] * (-dt / 2.0) + SS[e];
        for (int e = 0; e < 9; ++e) {
          SSo[e] = SSh[e];
          SSh[e] = X9[e] * dt + SSh[e];
        }
        target = SSh;
      } else {
        for (int e = 0; e < 9; ++e) {
          const double old = SS[e];
          SS[e] = (ct == 30) ? X9[e] * dt + SS[e] : X9[e] * (2.0 * dt) + SSh[e];
          SSh[e] = old;
        }
        target = SS;
      }
      if (C.fail == 1) {
        const double r = C.sigmay / sqrt(3.0 * J2of(target));
        const double f = (1.0 < r) ? 1.0 : r;
        for (int e = 0; e < 9; ++e) target[e] = target[e] * f;
      }
      if (lf)
        for (int e = 0; e < 9; ++e) SS[e] = (SSh[e] + SSo[e]) * (1.0 / 2.0);
      for (int e = 0; e < 9; ++e) Sig[e] = OIe(e) * -p + SS[e];
    } else {
      double* SS = P.shear ? P.shear + 9 * (size_t)s : nullptr;
      plane = (DIM == 2) && plane_zeros(SR, RR, Sig, Sh, E, Eh);
      if (plane) mat3_update<true>(C, I22, lf, first, ct, dt, SR, RR, Sig, Sh, So, SS);
      else mat3_update<false>(C, I22, lf, first, ct, dt, SR, RR, Sig, Sh, So, SS);
    }
    // strain integration (shared by Mat2 and Mat3)
    if (plane) strain_update<true>(lf, first, ct, dt, SR, E, Eh, Eo);
    else strain_update<false>(lf, first, ct, dt, SR, E, Eh, Eo);
  }
  // periodic wrap (Source/Particle.cpp:128-142) and CheckParticleLeave's test
  bool out = false;
  for (int d = 0; d < 3; ++d) {
    if (g.dom_size[d] > 0.0) {
      if (x[d] > g.trpr[d]) x[d] -= g.dom_size[d];
      if (x[d] < g.blpf[d]) x[d] += g.dom_size[d];
    }
    out |= (x[d] > g.trpr[d]) || (x[d] < g.blpf[d]);
  }
  if (DIM == 2) vel[2] = 0.0;  // StartAcceleration zeroes v_z in 2D (Source/Domain.cpp:1014)
  P.X4[s] = make_double4_32a(x[0], x[1], x[2], rho);
  P.V4[s] = make_double4_32a(vel[0], vel[1], vel[2], p);
  P.H4[s] = H;
  if (out) v.alive[s] = 0;
  if (o.skin > 0.f) {
    // neighbour lists with a skin: the largest displacement since the last
    // rebuild (from the FP32 position the sort recorded; both truncated on the
    // integer pipe, this kernel's FP64 pipe being its limit), and a particle
    // that left forces the next step to sort again
    float d2 = 0.f;
    if (v.S.cellid[s] >= 0) {
      const float4 r = v.S.OFFREF[s];
      const float e0 = d2f_bits(x[0]) - r.x, e1 = d2f_bits(x[1]) - r.y;
      const float e2 = (DIM == 3) ? d2f_bits(x[2]) - r.z : 0.f;
      d2 = e0 * e0 + e1 * e1 + e2 * e2;
    }
    if (out || !(d2 == d2)) atomicOr(&v.sc->force_rebuild, 1);
    const unsigned am = __activemask();
    const unsigned m = __reduce_max_sync(am, __float_as_uint(d2 == d2 ? d2 : 0.f));
    if ((int)(threadIdx.x & 31) == __ffs(am) - 1) atomicMax(&v.sc->disp2_bits, m);
  }
}

}  // namespace

void launch_update(const DevView& v, cudaStream_t st) {
  const int nb = (v.ncap + kUT - 1) / kUT;
  if (v.o.dim == 2) update_kernel<2><<<nb > 0 ? nb : 1, kUT, 0, st>>>(v);
  else update_kernel<3><<<nb > 0 ? nb : 1, kUT, 0, st>>>(v);
}

// begin, bin, 3 scan, scatter, rank, reorder (+ the solids' tensors), finish,
// cell starts, neighbour lists, prepare (2 in the FP32C form: copies + walls),
// forces, closure, dt, update, end
namespace {
__global__ void class_constants_kernel(PClass* cls, int n, int dim) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  PClass& C = cls[k];
  dp_constants(C.phi, C.coh, dim == 2 ? 0.0 : 1.0, &C.dp_alpha, &C.dp_kf);
  C.dp_sin_psi = sin(C.psi);
  C.eos_b = C.rho0 * C.cs * C.cs / 7.0;  // eos()'s expression for PresEq 1
  C.eos_inv_rho0 = 1.0 / C.rho0;
  C.eos_b32 = (float)C.eos_b;
}
}  // namespace

void launch_class_constants(PClass* cls, int n, int dim, cudaStream_t st) {
  if (n > 0) class_constants_kernel<<<(n + 127) / 128, 128, 0, st>>>(cls, n, dim);
}

namespace {
// Upload: the caller's arrays (copied as they are) into the persistent
// double4 layout, the particle's original index = its position.
__global__ void upload_pack_kernel(const double* __restrict__ sx, const double* __restrict__ sd,
                                   const double* __restrict__ sp, const double* __restrict__ sv,
                                   const double* __restrict__ sh1, const double* __restrict__ sh1s,
                                   const double* __restrict__ sh2, const double* __restrict__ sh2s,
                                   const double* __restrict__ smu, Persist P, int n, int two_d, int lf, int dyn_mu) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const size_t g3 = 3 * (size_t)g;
  P.X4[g] = make_double4_32a(sx[g3], sx[g3 + 1], sx[g3 + 2], sd[g]);
  P.V4[g] = make_double4_32a(sv[g3], sv[g3 + 1], two_d ? 0.0 : sv[g3 + 2], sp[g]);
  P.H4[g] = make_double4_32a(sh1[g3], sh1[g3 + 1], sh1[g3 + 2], sh1s[g]);
  if (lf) P.H4b[g] = make_double4_32a(sh2[g3], sh2[g3 + 1], sh2[g3 + 2], sh2s[g]);
  P.orig[g] = g;
  if (dyn_mu) P.mu[g] = smu[g];
}
}  // namespace

void launch_upload_pack(const double* sx, const double* sd, const double* sp, const double* sv, const double* sh1,
                        const double* sh1s, const double* sh2, const double* sh2s, const double* smu, const Persist& P,
                        int n, bool two_d, bool lf, bool dyn_mu, cudaStream_t st) {
  if (n > 0)
    upload_pack_kernel<<<(n + 255) / 256, 256, 0, st>>>(sx, sd, sp, sv, sh1, sh1s, sh2, sh2s, smu, P, n, two_d, lf,
                                                        dyn_mu);
}

int launches_per_step(const DevView& v) {
  return (v.o.fp32 ? 17 : 16) + (v.o.closure ? 1 : 0) + (v.o.has_solid ? 1 : 0) + (v.o.fp64_half ? 1 : 0) +
         (v.o.mixed ? 2 : 0) + (v.o.couple_soil && v.o.swi != 2 ? 2 : 0) + (v.o.fsi ? 1 : 0) +
         (v.o.skin > 0.f ? 1 : 0);
}

}  // namespace psph
