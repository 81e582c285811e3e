/*
 * CPU restatement of PersianSPH's per-step hot path: the parity ORACLE.
 * TEST INFRASTRUCTURE ONLY (see psph_oracle.h): never linked into the product.
 *
 * Each function restates one reference routine and cites it. Arithmetic is
 * written in the reference's own expression order (the blitz / matvec.h
 * element-wise operators evaluate per element in source order), so with
 * -ffp-contract=off the restatement reproduces the reference build bit for bit
 * on the same libm; the committed golden fixtures pin it.
 *
 * Differences from the reference, all outside its defined behaviour:
 *  - The acceleration dt minimum uses a proper reduction. The reference
 *    tests outside its lock (Source/Domain.cpp:1289-1294), which with Nproc>1
 *    can keep a larger value; with Nproc=1 both are the plain minimum.
 *  - A particle more than hmax outside the grid makes ListGenerate index out of
 *    bounds in the reference (Source/Domain.cpp:669-691); here it is an error.
 *  - Solid-soil pairs, which the reference aborts on, are reported as
 *    PSPH_ERR_INVALID_ARGUMENT.
 *  - The FSI interpolation's normalisation runs once per list entry of
 *    FreeFSIParticles, which holds a solid particle once per fluid pair
 *    (Source/Domain.cpp:1109, :1126, :1151-1157): the sums are divided by the
 *    kernel sum as many times, in sequence, as the reference does with
 *    Nproc = 1 (with more threads the duplicate entries race there).
 *  - Particle::n (porosity) is not kept: only the permeabilities it feeds are.
 */
#include "psph_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "state_io.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  int64_t* v; /* (first, second) couples */
  int64_t n, cap;
} pairvec;

struct psph_oracle {
  psph_config cfg;
  psph_grid g;
  psph_integrator it;
  double I[9]; /* Domain::I: identity, I(2,2)=0 in 2D (Source/Domain.cpp:1665) */
  int64_t n;
#define DECL_I(NAME) int32_t* NAME;
#define DECL_D(NAME) double* NAME;
  PSPH_INT_FIELDS(DECL_I)
  PSPH_F64_FIELDS(DECL_D)
  PSPH_VEC_FIELDS(DECL_D)
  PSPH_TEN_FIELDS(DECL_D)
  int64_t* orig;
  int32_t* LL; /* Particle::LL */
  int32_t* CC; /* Particle::CC[3] */
  int32_t* HOC;
  int32_t* satcheck; /* Particle::SatCheck of the current step */
  /* FSI interpolation of the current step (Particle::FSIPressure, FSINSv,
   * FSISumKernel) and the particle's entries in FreeFSIParticles */
  double *fsi_p, *fsi_nsv, *fsi_sk;
  int32_t* fsi_cnt;
  /* in/out-flow state (Domain::BC, Source/Boundary_Condition.h:38-60) */
  int inoutcounter;
  double in_loc1, in_loc2, in_loc3, out_loc;
  int64_t *in_part, n_in_part, cap_in_part; /* BC.InPart, in list order */
  int64_t n_out_part;                       /* BC.OutPart.Size() */
  int64_t next_orig;                        /* original index of the next appended particle */
  psph_flow_fn flow_fn[3];                  /* Domain::InCon / OutCon (NULL: InFlowCon / OutFlowCon) */
  void* flow_user[3];
  psph_oracle_hook_fn hook_fn;              /* Domain::GeneralBefore / GeneralAfter */
  void* hook_user;
  int hook_mask;
  int64_t ncells;
  int nthr;
  pairvec *sm, *fsm, *nsm;
  int64_t* fixed;
  int64_t nfixed;
  omp_lock_t* locks;
  double *a_scale, *dr_scale;
  double mu_max, cs_max; /* Domain::MuMax / CsMax from CellInitiate */
  double phase_s[5];
  int64_t pairs_done; /* in-support pairs evaluated by CalcForce* since create */
  int status;
  char err[512];
};

static int fail(psph_oracle* o, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(o->err, sizeof o->err, fmt, ap);
  va_end(ap);
  o->status = code;
  return code;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void pv_push(pairvec* p, int64_t a, int64_t b) {
  if (p->n + 1 > p->cap) {
    p->cap = p->cap ? 2 * p->cap : 1024;
    p->v = (int64_t*)realloc(p->v, (size_t)p->cap * 2 * sizeof(int64_t));
  }
  p->v[2 * p->n] = a;
  p->v[2 * p->n + 1] = b;
  p->n++;
}

/* ---------------------------------------------------------------------------
 * SPH functions (Source/Functions.cpp)
 * ------------------------------------------------------------------------- */

/* Kernel (Functions.cpp:25-63) */
static double Kernel(int Dim, int KT, double q, double h) {
  double C;
  switch (KT) {
    case 0:
      C = (Dim == 2) ? 10.0 / (7.0 * h * h * M_PI) : 1.0 / (h * h * h * M_PI);
      if (q < 1.0) return C * (1.0 - (3.0 / 2.0) * q * q + (3.0 / 4.0) * q * q * q);
      else if (q < 2.0) return C * ((1.0 / 4.0) * (2.0 - q) * (2.0 - q) * (2.0 - q));
      else return 0.0;
    case 1:
      C = (Dim == 2) ? 7.0 / (4.0 * h * h * M_PI) : 7.0 / (8.0 * h * h * h * M_PI);
      if (q < 2.0) return C * pow((1.0 - q / 2.0), 4.0) * (2.0 * q + 1.0);
      else return 0.0;
    default:
      C = (Dim == 2) ? 7.0 / (478.0 * h * h * M_PI) : 1.0 / (120.0 * h * h * h * M_PI);
      if (q < 1.0) return C * (pow((3.0 - q), 5.0) - 6.0 * pow((2.0 - q), 5.0) + 15.0 * pow((1.0 - q), 5.0));
      else if (q < 2.0) return C * (pow((3.0 - q), 5.0) - 6.0 * pow((2.0 - q), 5.0));
      else if (q < 3.0) return C * (pow((3.0 - q), 5.0));
      else return 0.0;
  }
}

/* GradKernel (Functions.cpp:65-106): (1/r) dW/dr */
static double GradKernel(int Dim, int KT, double q, double h) {
  double C;
  switch (KT) {
    case 0:
      C = (Dim == 2) ? 10.0 / (7.0 * h * h * h * M_PI) : 1.0 / (h * h * h * h * M_PI);
      if (q == 0.0) return C / h * (-3.0 + (9.0 / 2.0) * q);
      else if (q < 1.0) return C / (q * h) * (-3.0 * q + (9.0 / 4.0) * q * q);
      else if (q < 2.0) return C / (q * h) * ((-3.0 / 4.0) * (2.0 - q) * (2.0 - q));
      else return 0.0;
    case 1:
      C = (Dim == 2) ? 7.0 / (4.0 * h * h * h * M_PI) : 7.0 / (8.0 * h * h * h * h * M_PI);
      if (q == 0.0) return C * -5.0 / h * (pow((1.0 - q / 2.0), 3.0) - 3.0 * q / 2.0 * pow((1.0 - q / 2.0), 2.0));
      else if (q < 2.0) return C / (q * h) * -5.0 * q * pow((1.0 - q / 2.0), 3.0);
      else return 0.0;
    default:
      C = (Dim == 2) ? 7.0 / (478.0 * h * h * h * M_PI) : 1.0 / (120.0 * h * h * h * h * M_PI);
      if (q == 0.0)
        return C / h * (20.0 * pow((3.0 - q), 3.0) - 120.0 * pow((2.0 - q), 3.0) + 300.0 * pow((1.0 - q), 3.0));
      else if (q < 1.0)
        return C / (q * h) * (-5.0 * pow((3.0 - q), 4.0) + 30.0 * pow((2.0 - q), 4.0) - 75.0 * pow((1.0 - q), 4.0));
      else if (q < 2.0) return C / (q * h) * (-5.0 * pow((3.0 - q), 4.0) + 30.0 * pow((2.0 - q), 4.0));
      else if (q < 3.0) return C / (q * h) * (-5.0 * pow((3.0 - q), 4.0));
      else return 0.0;
  }
}

/* LaplaceKernel (Functions.cpp:108-146) */
static double LaplaceKernel(int Dim, int KT, double q, double h) {
  double C;
  switch (KT) {
    case 0:
      C = (Dim == 2) ? 10.0 / (7.0 * h * h * h * h * M_PI) : 1.0 / (h * h * h * h * h * M_PI);
      if (q < 1.0) return C * (-3.0 + (9.0 / 2.0) * q) + C * (Dim - 1.0) / q * (-3.0 * q + (9.0 / 4.0) * q * q);
      else if (q < 2.0)
        return C * ((3.0 / 2.0) * (2.0 - q)) + C * (Dim - 1.0) / q * ((-3.0 / 4.0) * (2.0 - q) * (2.0 - q));
      else return 0.0;
    case 1:
      C = (Dim == 2) ? 7.0 / (4.0 * h * h * h * h * M_PI) : 7.0 / (8.0 * h * h * h * h * h * M_PI);
      if (q < 2.0)
        return C * pow((1.0 - q / 2.0), 2.0) * (10.0 * q - 5.0) +
               C * (Dim - 1.0) / q * -5.0 * q * pow((1.0 - q / 2.0), 3.0);
      else return 0.0;
    default:
      C = (Dim == 2) ? 7.0 / (478.0 * h * h * h * h * M_PI) : 1.0 / (120.0 * h * h * h * h * h * M_PI);
      if (q < 1.0)
        return C * (20.0 * pow((3.0 - q), 3.0) - 120.0 * pow((2 - q), 3.0) + 300.0 * pow((1 - q), 3.0)) +
               C * (Dim - 1.0) / q *
                   (-5.0 * pow((3.0 - q), 4.0) + 30.0 * pow((2.0 - q), 4.0) - 75.0 * pow((1.0 - q), 4.0));
      else if (q < 2.0)
        return C * (20.0 * pow((3.0 - q), 3.0) - 120.0 * pow((2 - q), 3.0)) +
               C * (Dim - 1.0) / q * (-5.0 * pow((3.0 - q), 4.0) + 30.0 * pow((2.0 - q), 4.0));
      else if (q < 3.0)
        return C * (20.0 * pow((3.0 - q), 3.0)) + C * (Dim - 1.0) / q * (-5.0 * pow((3.0 - q), 4.0));
      else return 0.0;
  }
}

/* SecDerivativeKernel (Functions.cpp:148-186) */
static double SecDerivativeKernel(int Dim, int KT, double q, double h) {
  double C;
  switch (KT) {
    case 0:
      C = (Dim == 2) ? 10.0 / (7.0 * h * h * h * h * M_PI) : 1.0 / (h * h * h * h * h * M_PI);
      if (q < 1.0) return C * (-3.0 + (9.0 / 2.0) * q);
      else if (q < 2.0) return C * ((3.0 / 2.0) * (2.0 - q));
      else return 0.0;
    case 1:
      C = (Dim == 2) ? 7.0 / (4.0 * h * h * h * h * M_PI) : 7.0 / (8.0 * h * h * h * h * h * M_PI);
      if (q < 2.0) return C * pow((1.0 - q / 2.0), 2.0) * (10.0 * q - 5.0);
      else return 0.0;
    default:
      C = (Dim == 2) ? 7.0 / (478.0 * h * h * h * h * M_PI) : 1.0 / (120.0 * h * h * h * h * h * M_PI);
      if (q < 1.0) return C * (20.0 * pow((3.0 - q), 3.0) - 120.0 * pow((2.0 - q), 3.0) + 300.0 * pow((1.0 - q), 3.0));
      else if (q < 2.0) return C * (20.0 * pow((3.0 - q), 3.0) - 120.0 * pow((2.0 - q), 3.0));
      else if (q < 3.0) return C * (20.0 * pow((3.0 - q), 3.0));
      else return 0.0;
  }
}

/* EOS (Functions.cpp:188-212) */
static double EOS(int EQ, double Cs0, double P00, double Density, double Density0) {
  switch (EQ) {
    case 0: return P00 + (Cs0 * Cs0) * (Density - Density0);
    case 1: return P00 + (Density0 * Cs0 * Cs0 / 7.0) * (pow(Density / Density0, 7.0) - 1);
    default: return (Cs0 * Cs0) * Density;
  }
}

/* SoundSpeed (Functions.cpp:214-238) */
static double SoundSpeed(int EQ, double Cs0, double Density, double Density0) {
  switch (EQ) {
    case 1: return sqrt((Cs0 * Cs0) * pow(Density / Density0, 6.0));
    default: return Cs0;
  }
}

/* DensitySolid (Functions.cpp:240-264): inverse EOS */
static double DensitySolid(int EQ, double Cs0, double P00, double Pressure, double Density0) {
  switch (EQ) {
    case 0: return (Pressure - P00) / (Cs0 * Cs0) + Density0;
    case 1: return pow(((Pressure - P00) * (7.0 / (Density0 * Cs0 * Cs0)) + 1), 1.0 / 7.0) * Density0;
    default: return Pressure / (Cs0 * Cs0);
  }
}

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Viscous_Force (Functions.cpp:300-332) */
static void Viscous_Force(int VisEq, double* VI, double Mu, double di, double dj, double GK, const double* vab,
                          int Dim, int KT, double rij, double h, const double* xij, const double* vij) {
  switch (VisEq) {
    case 0: {
      double s = 2.0 * Mu / (di * dj) * GK;
      for (int d = 0; d < 3; ++d) VI[d] = s * vab[d];
    } break;
    case 1: {
      double s = 8.0 * Mu / ((di + dj) * (di + dj)) * GK;
      for (int d = 0; d < 3; ++d) VI[d] = s * vab[d];
    } break;
    case 2: {
      double s = -Mu / (di * dj) * LaplaceKernel(Dim, KT, rij / h, h);
      for (int d = 0; d < 3; ++d) VI[d] = s * vab[d];
    } break;
    default: {
      double L = LaplaceKernel(Dim, KT, rij / h, h);
      double S2 = SecDerivativeKernel(Dim, KT, rij / h, h);
      double dv = dot3(vij, xij);
      double s = -Mu / (di * dj);
      for (int d = 0; d < 3; ++d)
        VI[d] = s * (L * vab[d] + 1.0 / 3.0 * (GK * vij[d] + dv * xij[d] / (rij * rij) * (-GK + S2)));
    } break;
  }
}

/* ---------------------------------------------------------------------------
 * 3x3 helpers (External/matvec.h)
 * ------------------------------------------------------------------------- */
/* Mult(A,B,M) (matvec.h:814-820), the reference's own term order */
static void mat_mult(const double* A, const double* B, double* M) {
#define a(i, j) A[3 * (i) + (j)]
#define b(i, j) B[3 * (i) + (j)]
  M[0] = a(0, 2) * b(2, 0) + a(0, 1) * b(1, 0) + a(0, 0) * b(0, 0);
  M[1] = a(0, 2) * b(2, 1) + a(0, 1) * b(1, 1) + a(0, 0) * b(0, 1);
  M[2] = a(0, 2) * b(2, 2) + a(0, 1) * b(1, 2) + a(0, 0) * b(0, 2);
  M[3] = a(1, 2) * b(2, 0) + b(1, 0) * a(1, 1) + b(0, 0) * a(1, 0);
  M[4] = a(1, 2) * b(2, 1) + a(1, 1) * b(1, 1) + b(0, 1) * a(1, 0);
  M[5] = a(1, 2) * b(2, 2) + a(1, 1) * b(1, 2) + b(0, 2) * a(1, 0);
  M[6] = a(2, 2) * b(2, 0) + b(1, 0) * a(2, 1) + b(0, 0) * a(2, 0);
  M[7] = b(2, 1) * a(2, 2) + b(1, 1) * a(2, 1) + b(0, 1) * a(2, 0);
  M[8] = a(2, 2) * b(2, 2) + b(1, 2) * a(2, 1) + b(0, 2) * a(2, 0);
#undef a
#undef b
}
static void mat_trans(const double* M, double* T) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) T[3 * i + j] = M[3 * j + i];
}
static const double OI[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}; /* OrthoSys::I */

/* J2 of a deviatoric tensor, as Particle.cpp writes it (e.g. :363-365) */
static double J2of(const double* S) {
  return 0.5 * (S[0] * S[0] + 2.0 * S[1] * S[3] + 2.0 * S[2] * S[6] + S[4] * S[4] + 2.0 * S[5] * S[7] +
                S[8] * S[8]);
}

/* Cyclic Jacobi eigen-decomposition of a symmetric 3x3 (columns of Q are
 * eigenvectors), ascending eigenvalues: the Rotation() contract
 * (Functions.cpp:334-348 -> matvec.h:753-782 with SortAsc). */
static void sym_eig3(const double* Ain, double* val, double* Q) {
  double a[9];
  memcpy(a, Ain, sizeof a);
  for (int i = 0; i < 9; ++i) Q[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
    if (off == 0.0) break;
    for (int p = 0; p < 3; ++p)
      for (int r = p + 1; r < 3; ++r) {
        double apr = a[3 * p + r];
        if (apr == 0.0) continue;
        double theta = (a[3 * r + r] - a[3 * p + p]) / (2.0 * apr);
        double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = a[3 * k + p], akr = a[3 * k + r];
          a[3 * k + p] = c * akp - s * akr;
          a[3 * k + r] = s * akp + c * akr;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[3 * p + k], ark = a[3 * r + k];
          a[3 * p + k] = c * apk - s * ark;
          a[3 * r + k] = s * apk + c * ark;
        }
        for (int k = 0; k < 3; ++k) {
          double qkp = Q[3 * k + p], qkr = Q[3 * k + r];
          Q[3 * k + p] = c * qkp - s * qkr;
          Q[3 * k + r] = s * qkp + c * qkr;
        }
      }
  }
  for (int i = 0; i < 3; ++i) val[i] = a[4 * i];
  for (int i = 0; i < 2; ++i) { /* ascending selection sort */
    int b = i;
    for (int j = i + 1; j < 3; ++j)
      if (val[j] < val[b]) b = j;
    if (b != i) {
      double t = val[i];
      val[i] = val[b];
      val[b] = t;
      for (int k = 0; k < 3; ++k) {
        double u = Q[3 * k + i];
        Q[3 * k + i] = Q[3 * k + b];
        Q[3 * k + b] = u;
      }
    }
  }
}

/* Tensile-instability tensor TIR from Sigma (Source/Domain.cpp:955-987, repeated
 * for fixed particles at :1174-1204). */
static void tensile_tir(int dim, const double* S, double TI, double rho, double* TIR) {
  if (dim == 2) {
    double teta, Sxx, Syy, C, Sn;
    if ((S[0] - S[4]) != 0.0) teta = 0.5 * atan(2.0 * S[1] / (S[0] - S[4]));
    else teta = M_PI / 4.0;
    C = cos(teta);
    Sn = sin(teta);
    Sxx = C * C * S[0] + 2.0 * C * Sn * S[1] + Sn * Sn * S[4];
    Syy = Sn * Sn * S[0] - 2.0 * C * Sn * S[1] + C * C * S[4];
    if (Sxx > 0) Sxx = -TI * Sxx / (rho * rho); else Sxx = 0.0;
    if (Syy > 0) Syy = -TI * Syy / (rho * rho); else Syy = 0.0;
    TIR[0] = C * C * Sxx + Sn * Sn * Syy;
    TIR[4] = Sn * Sn * Sxx + C * C * Syy;
    TIR[1] = TIR[3] = Sn * C * (Sxx - Syy);
  } else {
    double val[3], Vec[9], VecT[9], Val[9] = {0}, tmp[9];
    sym_eig3(S, val, Vec);
    mat_trans(Vec, VecT);
    for (int k = 0; k < 3; ++k) Val[4 * k] = (val[k] > 0) ? -TI * val[k] / (rho * rho) : 0.0;
    mat_mult(Vec, Val, tmp);
    mat_mult(tmp, VecT, TIR);
  }
}

/* ---------------------------------------------------------------------------
 * Domain routines
 * ------------------------------------------------------------------------- */

#define FREE(p) (o->is_free[p] != 0)

/* Periodic_X_Correction (Source/Domain.cpp:110-115) */
static void periodic_correction(const psph_oracle* o, double* x, double h, int64_t p1, int64_t p2) {
  const double cf = o->g.cellfac;
  for (int d = 0; d < 3; ++d)
    if (o->g.dom_size[d] > 0.0)
      if (x[d] > 2 * cf * h || x[d] < -2 * cf * h) {
        if (o->CC[3 * p1 + d] > o->CC[3 * p2 + d]) x[d] -= o->g.dom_size[d];
        else x[d] += o->g.dom_size[d];
      }
}

/* CellInitiate (Source/Domain.cpp:549-660) */
static int cell_initiate(psph_oracle* o) {
  double TRPR[3] = {0, 0, 0}, BLPF[3] = {0, 0, 0};
  double hmax = 0, rhomax = 0;
  const double cf = o->g.cellfac;
  const int64_t n = o->n;
  if (n < 1) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "no particles");
  for (int d = 0; d < 3; ++d) BLPF[d] = TRPR[d] = o->x[d];
  hmax = o->h[0];
  rhomax = o->density[0];
  for (int64_t i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) {
      if (o->x[3 * i + d] > TRPR[d]) TRPR[d] = o->x[3 * i + d];
      if (o->x[3 * i + d] < BLPF[d]) BLPF[d] = o->x[3 * i + d];
    }
    if (o->h[i] > hmax) hmax = o->h[i];
    if (o->density[i] > rhomax) rhomax = o->density[i];
    if (o->mu[i] > o->mu_max) o->mu_max = o->mu[i];
    if (o->cs[i] > o->cs_max) o->cs_max = o->cs[i];
  }
  for (int d = 0; d < 3; ++d) {
    if (o->cfg.dom_max[d] > TRPR[d]) TRPR[d] = o->cfg.dom_max[d];
    if (o->cfg.dom_min[d] < BLPF[d]) BLPF[d] = o->cfg.dom_min[d];
  }
  for (int d = 0; d < 3; ++d) {
    if (!o->cfg.periodic[d]) {
      TRPR[d] += hmax / 2;
      BLPF[d] -= hmax / 2;
    } else {
      TRPR[d] += o->cfg.R;
      BLPF[d] -= o->cfg.R;
    }
  }
  int ndim = o->cfg.dimension;
  for (int d = 0; d < 3; ++d) {
    if (d < ndim) {
      double r = (TRPR[d] - BLPF[d]) / (cf * hmax);
      if ((double)(ceil(((TRPR[d] - BLPF[d]) / (cf * hmax))) - r) < (hmax / 10.0)) o->g.cell_no[d] = (int)ceil(r);
      else o->g.cell_no[d] = (int)floor(r);
      if (o->g.cell_no[d] < 1) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "domain thinner than one cell on axis %d", d);
      o->g.cell_size[d] = (TRPR[d] - BLPF[d]) / o->g.cell_no[d];
    } else {
      o->g.cell_no[d] = 1;
      o->g.cell_size[d] = 0.0;
    }
  }
  for (int d = 0; d < 3; ++d) {
    if (o->cfg.periodic[d]) o->g.cell_no[d] += 2;
    o->g.dom_size[d] = o->cfg.periodic[d] ? (TRPR[d] - BLPF[d]) : 0.0;
    o->g.blpf[d] = BLPF[d];
    o->g.trpr[d] = TRPR[d];
  }
  o->g.hmax = hmax;
  o->g.rhomax = rhomax;
  return PSPH_OK;
}

static int alloc_cells(psph_oracle* o) {
  o->ncells = (int64_t)o->g.cell_no[0] * o->g.cell_no[1] * o->g.cell_no[2];
  free(o->HOC);
  o->HOC = (int32_t*)malloc((size_t)o->ncells * sizeof(int32_t));
  if (!o->HOC) return fail(o, PSPH_ERR_OUT_OF_MEMORY, "HOC");
  for (int64_t c = 0; c < o->ncells; ++c) o->HOC[c] = -1;
  return PSPH_OK;
}

#define HOCI(o, i, j, k) ((o)->HOC[((int64_t)(i) * (o)->g.cell_no[1] + (j)) * (o)->g.cell_no[2] + (k)])

/* ListGenerate (Source/Domain.cpp:662-784) */
static int list_generate(psph_oracle* o) {
  const int dim = o->cfg.dimension;
  o->nfixed = 0;
  for (int64_t a = 0; a < o->n; ++a) {
    int c[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      const double xd = o->x[3 * a + d];
      c[d] = (int)(floor((xd - o->g.blpf[d]) / o->g.cell_size[d]));
      if (c[d] < 0) {
        if ((o->g.blpf[d] - xd) <= o->g.hmax) c[d] = 0;
        else return fail(o, PSPH_ERR_INVALID_ARGUMENT, "particle %lld left the grid (axis %d, low side)", (long long)o->orig[a], d);
      }
      if (c[d] >= o->g.cell_no[d]) {
        if ((xd - o->g.trpr[d]) <= o->g.hmax) c[d] = o->g.cell_no[d] - 1;
        else return fail(o, PSPH_ERR_INVALID_ARGUMENT, "particle %lld left the grid (axis %d, high side)", (long long)o->orig[a], d);
      }
    }
    int32_t temp = HOCI(o, c[0], c[1], c[2]);
    HOCI(o, c[0], c[1], c[2]) = (int32_t)a;
    o->LL[a] = temp;
    for (int d = 0; d < 3; ++d) o->CC[3 * a + d] = c[d];
    if (!FREE(a)) o->fixed[o->nfixed++] = a;
  }
  const int *N = o->g.cell_no;
  if (o->cfg.periodic[0])
    for (int j = 0; j < N[1]; j++)
      for (int k = 0; k < N[2]; k++) {
        HOCI(o, N[0] - 1, j, k) = HOCI(o, 1, j, k);
        HOCI(o, N[0] - 2, j, k) = HOCI(o, 0, j, k);
      }
  if (o->cfg.periodic[1])
    for (int i = 0; i < N[0]; i++)
      for (int k = 0; k < N[2]; k++) {
        HOCI(o, i, N[1] - 1, k) = HOCI(o, i, 1, k);
        HOCI(o, i, N[1] - 2, k) = HOCI(o, i, 0, k);
      }
  if (o->cfg.periodic[2])
    for (int i = 0; i < N[0]; i++)
      for (int j = 0; j < N[1]; j++) {
        HOCI(o, i, j, N[2] - 1) = HOCI(o, i, j, 1);
        HOCI(o, i, j, N[2] - 2) = HOCI(o, i, j, 0);
      }
  return PSPH_OK;
}

/* CellReset (Source/Domain.cpp:786-806) */
static void cell_reset(psph_oracle* o) {
  for (int64_t c = 0; c < o->ncells; ++c) o->HOC[c] = -1;
  for (int64_t a = 0; a < o->n; ++a) o->LL[a] = -1;
  o->nfixed = 0;
}

/* One candidate pair's classification (Source/Domain.cpp:844-856). */
static inline void classify(psph_oracle* o, int T, int64_t t1, int64_t t2) {
  if (FREE(t1) || FREE(t2)) {
    if (o->material[t1] == o->material[t2]) {
      if (FREE(t1) * FREE(t2)) pv_push(&o->sm[T], t1, t2);
      else pv_push(&o->fsm[T], t1, t2);
    } else
      pv_push(&o->nsm[T], t1, t2);
  }
}

/* YZPlaneCellsNeighbourSearch (Source/Domain.cpp:824-945) */
static void yz_plane_search(psph_oracle* o, int q1, int T) {
  const int *N = o->g.cell_no;
  const int *P = o->cfg.periodic;
  for (int q3 = P[2] ? 1 : 0; P[2] ? (q3 < (N[2] - 1)) : (q3 < N[2]); q3++)
    for (int q2 = P[1] ? 1 : 0; P[1] ? (q2 < (N[1] - 1)) : (q2 < N[1]); q2++) {
      if (HOCI(o, q1, q2, q3) == -1) continue;
      int32_t temp1 = HOCI(o, q1, q2, q3);
      while (temp1 != -1) {
        int32_t temp2 = o->LL[temp1];
        while (temp2 != -1) {
          classify(o, T, temp1, temp2);
          temp2 = o->LL[temp2];
        }
        if (q1 + 1 < N[0]) {
          temp2 = HOCI(o, q1 + 1, q2, q3);
          while (temp2 != -1) {
            classify(o, T, temp1, temp2);
            temp2 = o->LL[temp2];
          }
        }
        if (q2 + 1 < N[1]) {
          for (int i = q1 - 1; i <= q1 + 1; i++)
            if (i < N[0] && i >= 0) {
              temp2 = HOCI(o, i, q2 + 1, q3);
              while (temp2 != -1) {
                classify(o, T, temp1, temp2);
                temp2 = o->LL[temp2];
              }
            }
        }
        if (q3 + 1 < N[2]) {
          for (int j = q2 - 1; j <= q2 + 1; j++)
            for (int i = q1 - 1; i <= q1 + 1; i++)
              if (i < N[0] && i >= 0 && j < N[1] && j >= 0) {
                temp2 = HOCI(o, i, j, q3 + 1);
                while (temp2 != -1) {
                  classify(o, T, temp1, temp2);
                  temp2 = o->LL[temp2];
                }
              }
        }
        temp1 = o->LL[temp1];
      }
    }
}

/* MainNeighbourSearch (Source/Domain.cpp:808-822) */
static void main_search(psph_oracle* o, int nthr) {
  for (int t = 0; t < o->nthr; ++t) o->sm[t].n = o->fsm[t].n = o->nsm[t].n = 0;
  const int lo = o->cfg.periodic[0] ? 1 : 0;
  const int hi = o->cfg.periodic[0] ? o->g.cell_no[0] - 1 : o->g.cell_no[0];
#pragma omp parallel for schedule(dynamic) num_threads(nthr)
  for (int q1 = lo; q1 < hi; q1++) yz_plane_search(o, q1, omp_get_thread_num());
}

/* StartAcceleration (Source/Domain.cpp:947-1018) + the constant body force of
 * the GeneralBefore hook. */
static void start_acceleration(psph_oracle* o, int nthr) {
  const int dim = o->cfg.dimension;
  const double g0 = o->cfg.gravity[0], g1 = o->cfg.gravity[1], g2 = o->cfg.gravity[2];
  const double gn = sqrt(g0 * g0 + g1 * g1 + g2 * g2);
  const double* bf = o->cfg.body_force;
  const double bn = sqrt(bf[0] * bf[0] + bf[1] * bf[1] + bf[2] * bf[2]);
#pragma omp parallel for schedule(static) num_threads(nthr)
  for (int64_t i = 0; i < o->n; i++) {
    if (FREE(i)) {
      if (o->material[i] > 1 && o->ti[i] > 0.0) tensile_tir(dim, o->sigma + 9 * i, o->ti[i], o->density[i], o->tir + 9 * i);
    } else {
      for (int d = 0; d < 3; ++d) o->nsv[3 * i + d] = 0.0;
      o->pressure[i] = 0.0;
      memset(o->sigma + 9 * i, 0, 9 * sizeof(double));
      memset(o->shear_stress + 9 * i, 0, 9 * sizeof(double));
    }
    o->a[3 * i] = g0;
    o->a[3 * i + 1] = g1;
    o->a[3 * i + 2] = g2;
    o->ddensity[i] = 0.0;
    for (int d = 0; d < 3; ++d) o->vxsph[3 * i + d] = 0.0;
    o->zwab[i] = 0.0;
    o->sumden[i] = 0.0;
    o->sumkernel[i] = 0.0;
    o->satcheck[i] = 0;
    o->s[i] = 0.0;
    o->fsi_p[i] = 0.0;
    o->fsi_sk[i] = 0.0;
    o->fsi_cnt[i] = 0;
    for (int d = 0; d < 3; ++d) o->fsi_nsv[3 * i + d] = 0.0;
    if (dim == 2) o->v[3 * i + 2] = 0.0;
    memset(o->strain_rate + 9 * i, 0, 9 * sizeof(double));
    memset(o->rotation_rate + 9 * i, 0, 9 * sizeof(double));
    o->a_scale[i] = gn + (FREE(i) ? bn : 0.0);
    o->dr_scale[i] = 0.0;
    /* GeneralBefore: constant body force on free particles */
    if (FREE(i) && (bf[0] != 0.0 || bf[1] != 0.0 || bf[2] != 0.0))
      for (int d = 0; d < 3; ++d) o->a[3 * i + d] += bf[d];
  }
}

/* PrimaryComputeAcceleration, wall branch (Source/Domain.cpp:1020-1059,
 * normalisation and fixed-particle TIR :1164-1206). */
static void primary_compute(psph_oracle* o, int nthr) {
  const int dim = o->cfg.dimension, kt = o->cfg.kernel_type;
  const double* G = o->cfg.gravity;
  const int physical = o->cfg.wall_pressure_mode == PSPH_WALLP_PHYSICAL;
#pragma omp parallel for schedule(static) num_threads(nthr)
  for (int k = 0; k < o->nthr; k++) {
    for (int64_t a = 0; a < o->fsm[k].n; a++) {
      int64_t P1 = o->fsm[k].v[2 * a], P2 = o->fsm[k].v[2 * a + 1];
      double xij[3];
      for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * P1 + d] - o->x[3 * P2 + d];
      double h = (o->h[P1] + o->h[P2]) / 2.0;
      periodic_correction(o, xij, h, P1, P2);
      double K = Kernel(dim, kt, sqrt(dot3(xij, xij)) / h, h);
      int64_t W = FREE(P1) ? P2 : P1, F = FREE(P1) ? P1 : P2;
      double gx = dot3(G, xij);
      if (physical && W == P2) gx = -gx; /* x_wall - x_fluid */
      omp_set_lock(&o->locks[W]);
      o->sumkernel[W] += K;
      if (o->material[W] < 3) o->pressure[W] += o->pressure[F] * K + gx * o->density[F] * K;
      if (o->material[W] > 1)
        for (int e = 0; e < 9; ++e) o->sigma[9 * W + e] = o->sigma[9 * W + e] + o->sigma[9 * F + e] * K;
      if (o->no_slip[W])
        for (int d = 0; d < 3; ++d) o->nsv[3 * W + d] += o->v[3 * F + d] * K;
      omp_unset_lock(&o->locks[W]);
    }
    /* saturation check from the fluid-soil candidate pairs (Source/Domain.cpp:1060-1089):
     * a soil particle with a fluid particle in a neighbouring cell at or
     * above its own cell row and position is saturated this step */
    if (o->cfg.swi_type != 2)
      for (int64_t a = 0; a < o->nsm[k].n; a++) {
        int64_t P1 = o->nsm[k].v[2 * a], P2 = o->nsm[k].v[2 * a + 1];
        const int prod = o->material[P1] * o->material[P2];
        if (o->material[P1] == 3 && prod == 3)
          if (!o->satcheck[P1])
            if (o->CC[3 * P2 + 1] >= o->CC[3 * P1 + 1])
              if (o->x[3 * P2 + 1] >= o->x[3 * P1 + 1]) {
                omp_set_lock(&o->locks[P1]);
                o->satcheck[P1] = 1;
                omp_unset_lock(&o->locks[P1]);
              }
        if (o->material[P2] == 3 && prod == 3)
          if (!o->satcheck[P2])
            if (o->CC[3 * P1 + 1] >= o->CC[3 * P2 + 1])
              if (o->x[3 * P1 + 1] >= o->x[3 * P2 + 1]) {
                omp_set_lock(&o->locks[P2]);
                o->satcheck[P2] = 1;
                omp_unset_lock(&o->locks[P2]);
              }
      }
    /* FSI: a free solid particle interpolates pressure and velocity from its
     * free fluid candidates (Source/Domain.cpp:1090-1145); which sum the
     * velocity goes to, and the gravity term's sign, follow the pair's
     * orientation as in the reference */
    if (o->cfg.fsi)
      for (int64_t a = 0; a < o->nsm[k].n; a++) {
        int64_t P1 = o->nsm[k].v[2 * a], P2 = o->nsm[k].v[2 * a + 1];
        if (o->material[P1] * o->material[P2] != 2 || !(FREE(P1) * FREE(P2))) continue;
        double xij[3];
        for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * P1 + d] - o->x[3 * P2 + d];
        double h = (o->h[P1] + o->h[P2]) / 2.0;
        periodic_correction(o, xij, h, P1, P2);
        double K = Kernel(dim, kt, sqrt(dot3(xij, xij)) / h, h);
        const int64_t S = (o->material[P1] == 1) ? P2 : P1, F = (S == P1) ? P2 : P1;
        omp_set_lock(&o->locks[S]);
        o->fsi_cnt[S] += 1;
        o->fsi_sk[S] += K;
        if (S == P2)
          for (int d = 0; d < 3; ++d) o->nsv[3 * S + d] += o->v[3 * F + d] * K;
        else
          for (int d = 0; d < 3; ++d) o->fsi_nsv[3 * S + d] += o->v[3 * F + d] * K;
        o->fsi_p[S] += o->pressure[F] * K + dot3(G, xij) * o->density[F] * K;
        omp_unset_lock(&o->locks[S]);
      }
  }
  if (o->cfg.fsi) {
    /* Source/Domain.cpp:1147-1160, once per FreeFSIParticles entry */
#pragma omp parallel for schedule(static) num_threads(nthr)
    for (int64_t i = 0; i < o->n; i++)
      for (int32_t c = 0; c < o->fsi_cnt[i]; ++c) {
        o->fsi_p[i] = o->fsi_p[i] / o->fsi_sk[i];
        for (int d = 0; d < 3; ++d) o->fsi_nsv[3 * i + d] = o->fsi_nsv[3 * i + d] / o->fsi_sk[i];
      }
  }
#pragma omp parallel for schedule(static) num_threads(nthr)
  for (int64_t i = 0; i < o->nfixed; i++) {
    int64_t a = o->fixed[i];
    if (o->sumkernel[a] != 0.0) {
      if (o->material[a] < 3) o->pressure[a] = o->pressure[a] / o->sumkernel[a];
      if (o->material[a] > 1) {
        double s = 1.0 / o->sumkernel[a];
        for (int e = 0; e < 9; ++e) o->sigma[9 * a + e] = o->sigma[9 * a + e] * s;
      }
      if (o->no_slip[a])
        for (int d = 0; d < 3; ++d) o->nsv[3 * a + d] = o->nsv[3 * a + d] / o->sumkernel[a];
      if (o->material[a] > 1 && o->ti[a] > 0.0) tensile_tir(dim, o->sigma + 9 * a, o->ti[a], o->density[a], o->tir + 9 * a);
    }
  }
  /* saturated soil weighs its buoyant weight (Source/Domain.cpp:1209-1234) */
  if (o->cfg.swi_type != 2) {
#pragma omp parallel for schedule(static) num_threads(nthr)
    for (int64_t i = 0; i < o->n; i++)
      if (o->material[i] == 3) {
        if (o->satcheck[i] && !o->is_sat[i]) {
          o->mass[i] = o->volume[i] * (o->ref_density[i] - o->rho_f[i]);
          o->density[i] = o->density[i] - o->rho_f[i];
          o->densityb[i] = o->densityb[i] - o->rho_f[i];
          o->ref_density[i] = o->ref_density[i] - o->rho_f[i];
          o->is_sat[i] = 1;
        }
        if (!o->satcheck[i] && o->is_sat[i]) {
          o->mass[i] = o->volume[i] * (o->ref_density[i] + o->rho_f[i]);
          o->density[i] = o->density[i] + o->rho_f[i];
          o->densityb[i] = o->densityb[i] + o->rho_f[i];
          o->ref_density[i] = o->ref_density[i] + o->rho_f[i];
          o->is_sat[i] = 0;
        }
      }
  }
}

static inline double shepard_counter_of(const psph_oracle* o, int64_t p) {
  return FREE(p) ? o->it.shepard_counter : 0; /* fixed particles never move */
}

/* CalcForce11 (Source/Interaction.cpp:25-184) */
static int calc_force11(psph_oracle* o, int64_t p1, int64_t p2) {
  const int dim = o->cfg.dimension, kt = o->cfg.kernel_type;
  double h = (o->h[p1] + o->h[p2]) / 2;
  double xij[3];
  for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * p1 + d] - o->x[3 * p2 + d];
  periodic_correction(o, xij, h, p1, p2);
  double rij = sqrt(dot3(xij, xij));
  if ((rij / h) > o->g.cellfac) return 0;
  const int f1 = FREE(p1), f2 = FREE(p2);
  double di = 0.0, dj = 0.0, mi = 0.0, mj = 0.0;
  double Alpha = (o->alpha[p1] + o->alpha[p2]) / 2.0;
  double Beta = (o->beta[p1] + o->beta[p2]) / 2.0;
  double vij[3];
  for (int d = 0; d < 3; ++d) vij[d] = o->v[3 * p1 + d] - o->v[3 * p2 + d];
  if (!f1) {
    di = DensitySolid(o->pres_eq[p2], o->cs[p2], o->p0[p2], o->pressure[p1], o->ref_density[p2]);
    mi = o->fpmassc[p1] * o->mass[p2];
  } else {
    di = o->density[p1];
    mi = o->mass[p1];
  }
  if (!f2) {
    dj = DensitySolid(o->pres_eq[p1], o->cs[p1], o->p0[p1], o->pressure[p2], o->ref_density[p1]);
    mj = o->fpmassc[p2] * o->mass[p1];
  } else {
    dj = o->density[p2];
    mj = o->mass[p2];
  }
  double GK = GradKernel(dim, kt, rij / h, h);
  double K = Kernel(dim, kt, rij / h, h);

  double PIij = 0.0;
  if (Alpha != 0.0 || Beta != 0.0) {
    double Ci, Cj;
    if (!f1) Ci = SoundSpeed(o->pres_eq[p2], o->cs[p2], di, o->ref_density[p2]);
    else Ci = SoundSpeed(o->pres_eq[p1], o->cs[p1], di, o->ref_density[p1]);
    if (!f2) Cj = SoundSpeed(o->pres_eq[p1], o->cs[p1], dj, o->ref_density[p1]);
    else Cj = SoundSpeed(o->pres_eq[p2], o->cs[p2], dj, o->ref_density[p2]);
    double MUij = h * dot3(vij, xij) / (rij * rij + 0.01 * h * h);
    if (dot3(vij, xij) < 0) PIij = (-Alpha * 0.5 * (Ci + Cj) * MUij + Beta * MUij * MUij) / (0.5 * (di + dj));
  }

  double TIij = 0.0;
  if (o->ti[p1] > 0.0 || o->ti[p2] > 0.0) {
    double Ri = 0.0, Rj = 0.0;
    if ((o->pressure[p1] + o->pressure[p2]) < 0.0) {
      if (o->pressure[p1] < 0.0) Ri = -o->pressure[p1] / (di * di);
      if (o->pressure[p2] < 0.0) Rj = -o->pressure[p2] / (dj * dj);
    }
    TIij = (o->ti[p1] * Ri + o->ti[p2] * Rj) *
           pow((K / Kernel(dim, kt, (o->ti_init_dist[p1] + o->ti_init_dist[p2]) / (2.0 * h), h)),
               (o->tin[p1] + o->tin[p2]) / 2.0);
  }

  double SR[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double VI[3] = {0, 0, 0}, vab[3] = {0, 0, 0};
  const int want_sr = (o->t0[p1] > 0.0 || o->t0[p2] > 0.0 || (o->les[p1] * o->les[p2]));
  if ((o->no_slip[p1] || o->no_slip[p2]) || (f1 * f2)) {
    double Mu = 0.0;
    if (f1 * f2) {
      for (int d = 0; d < 3; ++d) vab[d] = vij[d];
      Mu = 2.0 * o->mu[p1] * o->mu[p2] / (o->mu[p1] + o->mu[p2]);
    } else {
      if (f1)
        for (int d = 0; d < 3; ++d) vab[d] = o->v[3 * p1 + d] - (2.0 * o->v[3 * p2 + d] - o->nsv[3 * p2 + d]);
      else
        for (int d = 0; d < 3; ++d) vab[d] = (2.0 * o->v[3 * p1 + d] - o->nsv[3 * p1 + d]) - o->v[3 * p2 + d];
      if (!f1) Mu = o->mu[p2];
      if (!f2) Mu = o->mu[p1];
    }
    if (want_sr) {
      SR[0] = 2.0 * vab[0] * xij[0];
      SR[1] = vab[0] * xij[1] + vab[1] * xij[0];
      SR[2] = vab[0] * xij[2] + vab[2] * xij[0];
      SR[3] = vab[0] * xij[1] + vab[1] * xij[0];
      SR[4] = 2.0 * vab[1] * xij[1];
      SR[5] = vab[1] * xij[2] + vab[2] * xij[1];
      SR[6] = vab[0] * xij[2] + vab[2] * xij[0];
      SR[7] = vab[1] * xij[2] + vab[2] * xij[1];
      SR[8] = 2.0 * vab[2] * xij[2];
      for (int e = 0; e < 9; ++e) SR[e] = SR[e] * -GK;
    }
    Viscous_Force(o->cfg.vis_eq, VI, Mu, di, dj, GK, vab, dim, kt, rij, h, xij, vij);
  }

  double X1[3] = {0, 0, 0}, X2[3] = {0, 0, 0};
  const int do_xsph = (o->cfg.xsph != 0.0 && (f1 * f2));
  if (do_xsph) {
    double s1 = o->cfg.xsph * mj / (0.5 * (di + dj)) * K, s2 = o->cfg.xsph * mi / (0.5 * (di + dj)) * K;
    for (int d = 0; d < 3; ++d) {
      X1[d] = s1 * -vij[d];
      X2[d] = s2 * vij[d];
    }
  }

  double temp[3], s;
  if (o->cfg.gradient_type == 0)
    s = -1.0 * (o->pressure[p1] / (di * di) + o->pressure[p2] / (dj * dj) + PIij + TIij) * GK;
  else
    s = -1.0 * ((o->pressure[p1] + o->pressure[p2]) / (di * dj) + PIij + TIij) * GK;
  for (int d = 0; d < 3; ++d) temp[d] = s * xij[d] + VI[d];
  if (dim == 2) temp[2] = 0.0;
  double gx[3] = {GK * xij[0], GK * xij[1], GK * xij[2]};
  double temp1 = dot3(vij, gx);
  const double tn = sqrt(dot3(temp, temp));

  omp_set_lock(&o->locks[p1]);
  for (int d = 0; d < 3; ++d) o->a[3 * p1 + d] += mj * temp[d];
  o->ddensity[p1] += mj * (di / dj) * temp1;
  if (do_xsph)
    for (int d = 0; d < 3; ++d) o->vxsph[3 * p1 + d] += X1[d];
  if (f1) {
    if (o->t0[p1] > 0.0 || o->les[p1]) {
      double c = mj / dj;
      for (int e = 0; e < 9; ++e) o->strain_rate[9 * p1 + e] = o->strain_rate[9 * p1 + e] + SR[e] * c;
    }
    if (o->cfg.swi_type == 1) o->s[p1] = o->s[p1] + mj / dj * vab[0] * xij[1] * -GK;
    o->zwab[p1] += mj / dj * K;
  } else
    o->zwab[p1] = 1.0;
  if (o->shepard[p1])
    if (shepard_counter_of(o, p1) == o->cfg.shepard_step) o->sumden[p1] += mj * K;
  o->a_scale[p1] += fabs(mj) * tn;
  o->dr_scale[p1] += fabs(mj * (di / dj) * temp1);
  omp_unset_lock(&o->locks[p1]);

  omp_set_lock(&o->locks[p2]);
  for (int d = 0; d < 3; ++d) o->a[3 * p2 + d] -= mi * temp[d];
  o->ddensity[p2] += mi * (dj / di) * temp1;
  if (do_xsph)
    for (int d = 0; d < 3; ++d) o->vxsph[3 * p2 + d] += X2[d];
  if (f2) {
    if (o->t0[p2] > 0.0 || o->les[p2]) {
      double c = mi / di;
      for (int e = 0; e < 9; ++e) o->strain_rate[9 * p2 + e] = o->strain_rate[9 * p2 + e] + SR[e] * c;
    }
    if (o->cfg.swi_type == 1) o->s[p2] = o->s[p2] + mi / di * vab[0] * xij[1] * -GK;
    o->zwab[p2] += mi / di * K;
  } else
    o->zwab[p2] = 1.0;
  if (o->shepard[p2])
    if (shepard_counter_of(o, p2) == o->cfg.shepard_step) o->sumden[p2] += mi * K;
  o->a_scale[p2] += fabs(mi) * tn;
  o->dr_scale[p2] += fabs(mi * (dj / di) * temp1);
  omp_unset_lock(&o->locks[p2]);
  return 1;
}

/* CalcForce2233 (Source/Interaction.cpp:186-377) */
static int calc_force2233(psph_oracle* o, int64_t p1, int64_t p2) {
  const int dim = o->cfg.dimension, kt = o->cfg.kernel_type;
  double h = (o->h[p1] + o->h[p2]) / 2;
  double xij[3];
  for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * p1 + d] - o->x[3 * p2 + d];
  periodic_correction(o, xij, h, p1, p2);
  double rij = sqrt(dot3(xij, xij));
  if ((rij / h) > o->g.cellfac) return 0;
  const int f1 = FREE(p1), f2 = FREE(p2);
  double di = 0.0, dj = 0.0, mi = 0.0, mj = 0.0;
  double Alpha = (o->alpha[p1] + o->alpha[p2]) / 2.0;
  double Beta = (o->beta[p1] + o->beta[p2]) / 2.0;
  const int soil = (o->material[p1] * o->material[p2] == 9);
  if (soil) {
    if (!f1) { di = o->density[p2]; mi = o->fpmassc[p1] * o->mass[p2]; } else { di = o->density[p1]; mi = o->mass[p1]; }
    if (!f2) { dj = o->density[p1]; mj = o->fpmassc[p2] * o->mass[p1]; } else { dj = o->density[p2]; mj = o->mass[p2]; }
  } else {
    if (!f1) {
      di = DensitySolid(o->pres_eq[p2], o->cs[p2], o->p0[p2], o->pressure[p1], o->ref_density[p2]);
      mi = o->fpmassc[p1] * o->mass[p2];
    } else {
      di = o->density[p1];
      mi = o->mass[p1];
    }
    if (!f2) {
      dj = DensitySolid(o->pres_eq[p1], o->cs[p1], o->p0[p1], o->pressure[p2], o->ref_density[p1]);
      mj = o->fpmassc[p2] * o->mass[p1];
    } else {
      dj = o->density[p2];
      mj = o->mass[p2];
    }
  }
  double vij[3];
  for (int d = 0; d < 3; ++d) vij[d] = o->v[3 * p1 + d] - o->v[3 * p2 + d];
  double GK = GradKernel(dim, kt, rij / h, h);
  double K = Kernel(dim, kt, rij / h, h);

  double PIij[9] = {0};
  if (Alpha != 0.0 || Beta != 0.0) {
    double MUij = h * dot3(vij, xij) / (rij * rij + 0.01 * h * h);
    double Cij;
    if (soil) Cij = 0.5 * (o->cs[p1] + o->cs[p2]);
    else {
      double Ci, Cj;
      if (!f1) Ci = SoundSpeed(o->pres_eq[p2], o->cs[p2], di, o->ref_density[p2]);
      else Ci = SoundSpeed(o->pres_eq[p1], o->cs[p1], di, o->ref_density[p1]);
      if (!f2) Cj = SoundSpeed(o->pres_eq[p1], o->cs[p1], dj, o->ref_density[p1]);
      else Cj = SoundSpeed(o->pres_eq[p2], o->cs[p2], dj, o->ref_density[p2]);
      Cij = 0.5 * (Ci + Cj);
    }
    if (dot3(vij, xij) < 0) {
      double s = (Alpha * Cij * MUij + Beta * MUij * MUij) / (0.5 * (di + dj));
      for (int e = 0; e < 9; ++e) PIij[e] = o->I[e] * s;
    }
  }
  const double* Sigmai = o->sigma + 9 * p1;
  const double* Sigmaj = o->sigma + 9 * p2;
  double TIij[9] = {0};
  if (o->ti[p1] > 0.0 || o->ti[p2] > 0.0) {
    double s = pow((K / Kernel(dim, kt, (o->ti_init_dist[p1] + o->ti_init_dist[p2]) / (2.0 * h), h)),
                   (o->tin[p1] + o->tin[p2]) / 2.0);
    for (int e = 0; e < 9; ++e) TIij[e] = (o->tir[9 * p1 + e] + o->tir[9 * p2 + e]) * s;
  }
  double vab[3] = {0, 0, 0};
  if (f1 * f2) {
    for (int d = 0; d < 3; ++d) vab[d] = vij[d];
  } else {
    const int ns = o->no_slip[p1] || o->no_slip[p2];
    if (ns) {
      if (f1)
        for (int d = 0; d < 3; ++d) vab[d] = o->v[3 * p1 + d] - (2.0 * o->v[3 * p2 + d] - o->nsv[3 * p2 + d]);
      else
        for (int d = 0; d < 3; ++d) vab[d] = (2.0 * o->v[3 * p1 + d] - o->nsv[3 * p1 + d]) - o->v[3 * p2 + d];
    }
    if (!ns) {
      if (f1)
        for (int d = 0; d < 3; ++d) vab[d] = o->v[3 * p1 + d] - o->vb[3 * p2 + d];
      else
        for (int d = 0; d < 3; ++d) vab[d] = o->vb[3 * p1 + d] - o->v[3 * p2 + d];
    }
  }
  double SR[9], RR[9] = {0};
  SR[0] = 2.0 * vab[0] * xij[0];
  SR[1] = vab[0] * xij[1] + vab[1] * xij[0];
  SR[2] = vab[0] * xij[2] + vab[2] * xij[0];
  SR[3] = SR[1];
  SR[4] = 2.0 * vab[1] * xij[1];
  SR[5] = vab[1] * xij[2] + vab[2] * xij[1];
  SR[6] = SR[2];
  SR[7] = SR[5];
  SR[8] = 2.0 * vab[2] * xij[2];
  double sc = -0.5 * GK;
  for (int e = 0; e < 9; ++e) SR[e] = SR[e] * sc;
  RR[1] = vab[0] * xij[1] - vab[1] * xij[0];
  RR[2] = vab[0] * xij[2] - vab[2] * xij[0];
  RR[5] = vab[1] * xij[2] - vab[2] * xij[1];
  RR[3] = -RR[1];
  RR[6] = -RR[2];
  RR[7] = -RR[5];
  for (int e = 0; e < 9; ++e) RR[e] = RR[e] * sc;

  double X1[3] = {0, 0, 0}, X2[3] = {0, 0, 0};
  const int do_xsph = (o->cfg.xsph != 0.0 && (f1 * f2));
  if (do_xsph) {
    double s1 = o->cfg.xsph * mj / (0.5 * (di + dj)) * K, s2 = o->cfg.xsph * mi / (0.5 * (di + dj)) * K;
    for (int d = 0; d < 3; ++d) {
      X1[d] = s1 * -vij[d];
      X2[d] = s2 * vij[d];
    }
  }

  double M[9], temp[3];
  if (o->cfg.gradient_type == 0) {
    double ci = 1.0 / (di * di), cj = 1.0 / (dj * dj);
    for (int e = 0; e < 9; ++e) M[e] = ((Sigmai[e] * ci + Sigmaj[e] * cj) + PIij[e]) + TIij[e];
  } else {
    double c = 1.0 / (di * dj);
    for (int e = 0; e < 9; ++e) M[e] = ((Sigmai[e] + Sigmaj[e]) * c + PIij[e]) + TIij[e];
  }
  double gx[3] = {GK * xij[0], GK * xij[1], GK * xij[2]};
  for (int c = 0; c < 3; ++c) temp[c] = gx[0] * M[c] + gx[1] * M[3 + c] + gx[2] * M[6 + c]; /* Mult(Vec,Mat) */
  if (dim == 2) temp[2] = 0.0;
  double temp1 = dot3(vij, gx);
  const double tn = sqrt(dot3(temp, temp));

  omp_set_lock(&o->locks[p1]);
  for (int d = 0; d < 3; ++d) o->a[3 * p1 + d] += mj * temp[d];
  o->ddensity[p1] += mj * (di / dj) * temp1;
  if (do_xsph)
    for (int d = 0; d < 3; ++d) o->vxsph[3 * p1 + d] += X1[d];
  if (f1) {
    o->zwab[p1] += mj / dj * K;
    double c = mj / dj;
    for (int e = 0; e < 9; ++e) {
      o->strain_rate[9 * p1 + e] = o->strain_rate[9 * p1 + e] + SR[e] * c;
      o->rotation_rate[9 * p1 + e] = o->rotation_rate[9 * p1 + e] + RR[e] * c;
    }
    if (o->cfg.swi_type == 1) o->s[p1] = o->s[p1] + mj / dj * vab[0] * xij[1] * -GK;
  } else
    o->zwab[p1] = 1.0;
  if (o->shepard[p1])
    if (shepard_counter_of(o, p1) == o->cfg.shepard_step) o->sumden[p1] += mj * K;
  o->a_scale[p1] += fabs(mj) * tn;
  o->dr_scale[p1] += fabs(mj * (di / dj) * temp1);
  omp_unset_lock(&o->locks[p1]);

  omp_set_lock(&o->locks[p2]);
  for (int d = 0; d < 3; ++d) o->a[3 * p2 + d] -= mi * temp[d];
  o->ddensity[p2] += mi * (dj / di) * temp1;
  if (do_xsph)
    for (int d = 0; d < 3; ++d) o->vxsph[3 * p2 + d] += X2[d];
  if (f2) {
    o->zwab[p2] += mi / di * K;
    double c = mi / di;
    for (int e = 0; e < 9; ++e) {
      o->strain_rate[9 * p2 + e] = o->strain_rate[9 * p2 + e] + SR[e] * c;
      o->rotation_rate[9 * p2 + e] = o->rotation_rate[9 * p2 + e] + RR[e] * c;
    }
    if (o->cfg.swi_type == 1) o->s[p2] = o->s[p2] + mi / di * vab[0] * xij[1] * -GK;
  } else
    o->zwab[p2] = 1.0;
  if (o->shepard[p2])
    if (shepard_counter_of(o, p2) == o->cfg.shepard_step) o->sumden[p2] += mi * K;
  o->a_scale[p2] += fabs(mi) * tn;
  o->dr_scale[p2] += fabs(mi * (dj / di) * temp1);
  omp_unset_lock(&o->locks[p2]);
  return 1;
}

/* CalcForce12 (Source/Interaction.cpp:379-507): fluid-solid pair. The solid
 * side enters with the density its interpolated FSIPressure gives under the
 * fluid's EOS, the fluid's mass on both sides and the no-slip velocity from
 * FSINSv; the reference's artificial-viscosity branch is dead (Alpha and Beta
 * are set to zero just before their test), and the solid gets no density rate
 * or strain rate. */
static int calc_force12(psph_oracle* o, int64_t p1, int64_t p2) {
  const int dim = o->cfg.dimension, kt = o->cfg.kernel_type;
  double h = (o->h[p1] + o->h[p2]) / 2;
  double xij[3];
  for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * p1 + d] - o->x[3 * p2 + d];
  periodic_correction(o, xij, h, p1, p2);
  double rij = sqrt(dot3(xij, xij));
  if ((rij / h) > o->g.cellfac) return 0;
  double di, dj, mi, mj, vij[3];
  for (int d = 0; d < 3; ++d) vij[d] = o->v[3 * p1 + d] - o->v[3 * p2 + d];
  double GK = GradKernel(dim, kt, rij / h, h);
  const int fluid1 = (o->material[p1] == 1);
  if (fluid1) {
    di = o->density[p1];
    mi = o->mass[p1];
    dj = DensitySolid(o->pres_eq[p1], o->cs[p1], o->p0[p1], o->fsi_p[p2], o->ref_density[p1]);
    mj = o->mass[p1];
  } else {
    di = DensitySolid(o->pres_eq[p2], o->cs[p2], o->p0[p2], o->fsi_p[p1], o->ref_density[p2]);
    mi = o->mass[p2];
    dj = o->density[p2];
    mj = o->mass[p2];
  }
  const double PIij = 0.0;
  double SR[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, VI[3] = {0, 0, 0}, vab[3], Mu;
  if (fluid1) {
    for (int d = 0; d < 3; ++d) vab[d] = o->v[3 * p1 + d] - (2.0 * o->v[3 * p2 + d] - o->fsi_nsv[3 * p2 + d]);
    Mu = o->mu[p1];
  } else {
    for (int d = 0; d < 3; ++d) vab[d] = (2.0 * o->v[3 * p1 + d] - o->fsi_nsv[3 * p1 + d]) - o->v[3 * p2 + d];
    Mu = o->mu[p2];
  }
  if ((o->t0[p1] > 0.0 || o->t0[p2] > 0.0) || (o->les[p1] || o->les[p2])) {
    SR[0] = 2.0 * vab[0] * xij[0];
    SR[1] = vab[0] * xij[1] + vab[1] * xij[0];
    SR[2] = vab[0] * xij[2] + vab[2] * xij[0];
    SR[3] = vab[0] * xij[1] + vab[1] * xij[0];
    SR[4] = 2.0 * vab[1] * xij[1];
    SR[5] = vab[1] * xij[2] + vab[2] * xij[1];
    SR[6] = vab[0] * xij[2] + vab[2] * xij[0];
    SR[7] = vab[1] * xij[2] + vab[2] * xij[1];
    SR[8] = 2.0 * vab[2] * xij[2];
    for (int e = 0; e < 9; ++e) SR[e] = SR[e] * -GK;
  }
  Viscous_Force(o->cfg.vis_eq, VI, Mu, di, dj, GK, vab, dim, kt, rij, h, xij, vij);
  const double p1v = fluid1 ? o->pressure[p1] : o->fsi_p[p1];
  const double p2v = fluid1 ? o->fsi_p[p2] : o->pressure[p2];
  double s;
  if (o->cfg.gradient_type == 0) s = -1.0 * (p1v / (di * di) + p2v / (dj * dj) + PIij) * GK;
  else s = -1.0 * ((p1v + p2v) / (di * dj) + PIij) * GK;
  double temp[3];
  for (int d = 0; d < 3; ++d) temp[d] = s * xij[d] + VI[d];
  if (dim == 2) temp[2] = 0.0;
  double gx[3] = {GK * xij[0], GK * xij[1], GK * xij[2]};
  double temp1 = dot3(vij, gx);
  const double tn = sqrt(dot3(temp, temp));
  omp_set_lock(&o->locks[p1]);
  for (int d = 0; d < 3; ++d) o->a[3 * p1 + d] += mj * temp[d];
  if (fluid1) {
    o->ddensity[p1] += mj * (di / dj) * temp1;
    if (o->t0[p1] > 0.0 || o->les[p1]) {
      double c = mj / dj;
      for (int e = 0; e < 9; ++e) o->strain_rate[9 * p1 + e] = o->strain_rate[9 * p1 + e] + SR[e] * c;
    }
    o->dr_scale[p1] += fabs(mj * (di / dj) * temp1);
  }
  o->a_scale[p1] += fabs(mj) * tn;
  omp_unset_lock(&o->locks[p1]);
  omp_set_lock(&o->locks[p2]);
  for (int d = 0; d < 3; ++d) o->a[3 * p2 + d] -= mi * temp[d];
  if (!fluid1) {
    o->ddensity[p2] += mi * (dj / di) * temp1;
    if (o->t0[p2] > 0.0 || o->les[p2]) {
      double c = mi / di;
      for (int e = 0; e < 9; ++e) o->strain_rate[9 * p2 + e] = o->strain_rate[9 * p2 + e] + SR[e] * c;
    }
    o->dr_scale[p2] += fabs(mi * (dj / di) * temp1);
  }
  o->a_scale[p2] += fabs(mi) * tn;
  omp_unset_lock(&o->locks[p2]);
  return 1;
}

/* Seepage (Source/Functions.cpp:266-298): Darcy (0, 1) or Forchheimer (2, 3)
 * coefficients of the drag between pore fluid and soil skeleton */
static void Seepage(int ST, double k, double k2, double mu, double rho, double* SF1, double* SF2) {
  *SF1 = mu / k;
  *SF2 = (ST >= 2) ? k2 * rho : 0.0;
}

/* CalcForce13 (Source/Interaction.cpp:508-653): fluid-soil pair. Both of the
 * reference's orientations give the same terms (v = v_fluid - v_soil; the
 * pore-pressure term's sign follows x_ij), written here from the soil side. */
static int calc_force13(psph_oracle* o, int64_t p1, int64_t p2) {
  const int dim = o->cfg.dimension, kt = o->cfg.kernel_type;
  double h = o->h[p1] < o->h[p2] ? o->h[p1] : o->h[p2];
  double xij[3];
  for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * p1 + d] - o->x[3 * p2 + d];
  periodic_correction(o, xij, h, p1, p2);
  double rij = sqrt(dot3(xij, xij));
  if ((rij / h) > o->g.cellfac) return 0;
  const int swi = o->cfg.swi_type;
  if (swi == 3) return 1;
  double K = Kernel(dim, kt, rij / h, h) / (o->density[p1] * o->density[p2]);
  const int64_t S = (o->material[p1] == 3) ? p1 : p2, F = (S == p1) ? p2 : p1;
  double v[3], SF1 = 0.0, SF2 = 0.0, SFt[3];
  for (int d = 0; d < 3; ++d) v[d] = o->v[3 * F + d] - o->v[3 * S + d];
  const double nv = sqrt(dot3(v, v));
  if (swi == 1 && o->zwab[S] < 0.25) {
    /* surface erosion: drag of a grain at the soil surface plus lift from the
     * fluid's velocity derivative (Source/Interaction.cpp:561-566) */
    double Cd = 24.0 * (o->mu_ref[F] / o->ref_density[F]) / (o->d[S] * nv + 0.01 * h * h) + 2.0;
    double c = 3.0 / (4.0 * o->d[S]) * o->ref_density[F] * (1.0 - o->n0[S]) * Cd * nv;
    for (int d = 0; d < 3; ++d) SFt[d] = c * v[d] * K;
    SFt[1] += (o->ref_density[F] * (1.0 - o->n0[S]) * nv * fabs(o->s[F] - o->s[S])) * K;
  } else {
    Seepage(o->seepage_type[S], o->k[S], o->k2[S], o->mu_ref[F], o->ref_density[F], &SF1, &SF2);
    for (int d = 0; d < 3; ++d) SFt[d] = (SF1 * v[d] + SF2 * nv * v[d]) * K;
  }
  if (dim == 2) SFt[2] = 0.0;
  double as[3];
  for (int d = 0; d < 3; ++d) as[d] = o->mass[F] * SFt[d];
  if (swi == 2) {
    /* pore pressure of the fluid on the soil (Source/Interaction.cpp:608-637) */
    double GK = GradKernel(dim, kt, rij / h, h) / (o->density[p1] * o->density[p2]);
    double c = o->mass[F] * o->pressure[F] * GK;
    for (int d = 0; d < 3; ++d) as[d] = (S == p1) ? as[d] - c * xij[d] : as[d] + c * xij[d];
  }
  const double tf = o->mass[S] * sqrt(dot3(SFt, SFt)), ts = sqrt(dot3(as, as));
  omp_set_lock(&o->locks[S]);
  for (int d = 0; d < 3; ++d) o->a[3 * S + d] += as[d];
  o->a_scale[S] += ts;
  omp_unset_lock(&o->locks[S]);
  omp_set_lock(&o->locks[F]);
  for (int d = 0; d < 3; ++d) o->a[3 * F + d] -= o->mass[S] * SFt[d];
  o->a_scale[F] += tf;
  omp_unset_lock(&o->locks[F]);
  return 1;
}

/* LastComputeAcceleration (Source/Domain.cpp:1238-1297) */
static int last_compute(psph_oracle* o, int nthr) {
  for (int k = 0; k < o->nthr; ++k)
    for (int64_t i = 0; i < o->nsm[k].n; i++) {
      const int prod = o->material[o->nsm[k].v[2 * i]] * o->material[o->nsm[k].v[2 * i + 1]];
      if (prod != 2 && prod != 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Out of Interaction types");
    }
  int64_t evaluated = 0;
#pragma omp parallel for schedule(static) num_threads(nthr) reduction(+ : evaluated)
  for (int k = 0; k < o->nthr; k++) {
    for (int64_t i = 0; i < o->sm[k].n; i++) {
      int64_t p1 = o->sm[k].v[2 * i], p2 = o->sm[k].v[2 * i + 1];
      evaluated += (o->material[p1] == 1) ? calc_force11(o, p1, p2) : calc_force2233(o, p1, p2);
    }
    for (int64_t i = 0; i < o->fsm[k].n; i++) {
      int64_t p1 = o->fsm[k].v[2 * i], p2 = o->fsm[k].v[2 * i + 1];
      evaluated += (o->material[p1] == 1) ? calc_force11(o, p1, p2) : calc_force2233(o, p1, p2);
    }
  }
#pragma omp parallel for schedule(static) num_threads(nthr) reduction(+ : evaluated)
  for (int k = 0; k < o->nthr; k++)
    for (int64_t i = 0; i < o->nsm[k].n; i++) {
      int64_t p1 = o->nsm[k].v[2 * i], p2 = o->nsm[k].v[2 * i + 1];
      evaluated += (o->material[p1] * o->material[p2] == 3) ? calc_force13(o, p1, p2) : calc_force12(o, p1, p2);
    }
  o->pairs_done += evaluated;
  double dtmin = o->it.deltatint;
  const double sha = o->cfg.sqrt_h_a;
#pragma omp parallel for schedule(static) num_threads(nthr) reduction(min : dtmin)
  for (int64_t i = 0; i < o->n; i++)
    if (FREE(i)) {
      const double* a = o->a + 3 * i;
      double test = sqrt(o->h[i] / sqrt(dot3(a, a)));
      if (dtmin > (sha * test)) dtmin = sha * test;
    }
  o->it.deltatmin = dtmin;
  return PSPH_OK;
}

/* AdaptiveTimeStep (Source/Domain.cpp:133-152) */
static int adaptive_time_step(psph_oracle* o) {
  psph_integrator* t = &o->it;
  if (t->deltatint > t->deltatmin) {
    if (t->deltat < t->deltatmin) t->deltat = 2.0 * t->deltat * t->deltatmin / (t->deltat + t->deltatmin);
    else t->deltat = t->deltatmin;
  } else {
    if (t->deltatint != t->deltat) t->deltat = 2.0 * t->deltat * t->deltatint / (t->deltat + t->deltatint);
    else t->deltat = t->deltatint;
  }
  if (t->deltat < (t->deltatint / 1.0e5))
    return fail(o, PSPH_ERR_DT_COLLAPSE, "Too small time step, please choose a smaller time step initially to make the simulation more stable");
  return PSPH_OK;
}

/* Mat1 (Source/Particle.cpp:146-186) */
static void mat1(psph_oracle* o, int64_t i) {
  o->pressure[i] = EOS(o->pres_eq[i], o->cs[i], o->p0[i], o->density[i], o->ref_density[i]);
  const double* S = o->strain_rate + 9 * i;
  double temp = (S[0] * S[0] + 2.0 * S[1] * S[3] + 2.0 * S[2] * S[6] + S[4] * S[4] + 2.0 * S[5] * S[7] + S[8] * S[8]);
  o->shear_rate[i] = sqrt(0.5 * temp);
  o->sbar[i] = sqrt(2.0 * temp);
  if (o->les[i]) o->mu[i] = o->mu_ref[i] + o->ref_density[i] * pow((o->csmag[i] * o->h[i]), 2.0) * o->sbar[i];
  if (o->t0[i] > 0.0) {
    const double sr = o->shear_rate[i], T0 = o->t0[i], MuRef = o->mu_ref[i], m = o->bingham_m[i];
    if (o->vis_m[i] == 0) {
      if (sr != 0.0) o->mu[i] = MuRef + T0 * (1 - exp(-m * sr)) / sr;
      else o->mu[i] = MuRef + T0 * m;
    } else
      o->mu[i] = (1000.0 * MuRef + MuRef * MuRef * 1000.0 / T0 * sr) / (1 + 1000.0 * MuRef / T0 * sr);
  }
}

/* Deviatoric elastic rate 2G(D - tr(D)/3 I) + S W^T + W S, the bracket of
 * Particle.cpp:286-289 / :614-617 (solid, around ShearStress). */
static void mat2_rate(const double* SR, const double* RR, const double* SS, double G, double* X) {
  double RRT[9], SRT[9], RS[9];
  mat_trans(RR, RRT);
  mat_mult(SS, RRT, SRT);
  mat_mult(RR, SS, RS);
  double s_tr = 1.0 / 3.0 * (SR[0] + SR[4] + SR[8]);
  double g2 = 2.0 * G;
  for (int e = 0; e < 9; ++e) X[e] = (((SR[e] - OI[e] * s_tr) * g2) + SRT[e]) + RS[e];
}

/* Elastic stress rate K tr(D) I + 2G(D - tr(D)/3 I) + Sigma W^T + W Sigma
 * (Particle.cpp:337-339 / :659-661, soil, around Sigma). */
static void mat3_rate(const double* SR, const double* RR, const double* Sig, double K, double G, double* X) {
  double RRT[9], SRT[9], RS[9];
  mat_trans(RR, RRT);
  mat_mult(Sig, RRT, SRT);
  mat_mult(RR, Sig, RS);
  double I1s = SR[0] + SR[4] + SR[8];
  double sK = I1s * K, s3 = 1.0 / 3.0 * I1s, g2 = 2.0 * G;
  for (int e = 0; e < 9; ++e) X[e] = ((OI[e] * sK + ((SR[e] - OI[e] * s3) * g2)) + SRT[e]) + RS[e];
}

/* Mat2Leapfrog (Particle.cpp:598-639) */
static int mat2_leapfrog(psph_oracle* o, int64_t i, double dt) {
  o->pressure[i] = EOS(o->pres_eq[i], o->cs[i], o->p0[i], o->density[i], o->ref_density[i]);
  double *SS = o->shear_stress + 9 * i, *Sa = o->shear_stressa + 9 * i, *Sb = o->shear_stressb + 9 * i;
  const double *SR = o->strain_rate + 9 * i, *RR = o->rotation_rate + 9 * i;
  double X[9];
  mat2_rate(SR, RR, SS, o->g_mod[i], X);
  if (o->it.first_step)
    for (int e = 0; e < 9; ++e) Sa[e] = X[e] * (-dt / 2.0) + SS[e];
  for (int e = 0; e < 9; ++e) Sb[e] = Sa[e];
  for (int e = 0; e < 9; ++e) Sa[e] = X[e] * dt + Sa[e];
  if (o->fail[i] == 1) {
    double J2 = J2of(Sa);
    double r = o->sigmay[i] / sqrt(3.0 * J2);
    double s = (1.0 < r) ? 1.0 : r; /* std::min(r, 1.0) */
    for (int e = 0; e < 9; ++e) Sa[e] = Sa[e] * s;
  }
  for (int e = 0; e < 9; ++e) SS[e] = (Sa[e] + Sb[e]) * (1.0 / 2.0);
  double* Sig = o->sigma + 9 * i;
  for (int e = 0; e < 9; ++e) Sig[e] = OI[e] * -o->pressure[i] + SS[e];
  double *E = o->strain + 9 * i, *Ea = o->straina + 9 * i, *Eb = o->strainb + 9 * i;
  if (o->it.first_step)
    for (int e = 0; e < 9; ++e) Ea[e] = SR[e] * (-dt / 2.0) + E[e];
  for (int e = 0; e < 9; ++e) Eb[e] = Ea[e];
  for (int e = 0; e < 9; ++e) Ea[e] = SR[e] * dt + Ea[e];
  for (int e = 0; e < 9; ++e) E[e] = (Ea[e] + Eb[e]) * (1.0 / 2.0);
  if (o->fail[i] > 1) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Undefined failure criteria for solids");
  return PSPH_OK;
}

/* Mat2MVerlet (Particle.cpp:276-318) */
static int mat2_mverlet(psph_oracle* o, int64_t i, double dt, int ct) {
  o->pressure[i] = EOS(o->pres_eq[i], o->cs[i], o->p0[i], o->density[i], o->ref_density[i]);
  double *SS = o->shear_stress + 9 * i, *Sb = o->shear_stressb + 9 * i;
  const double *SR = o->strain_rate + 9 * i, *RR = o->rotation_rate + 9 * i;
  double X[9], Stress[9];
  mat2_rate(SR, RR, SS, o->g_mod[i], X);
  memcpy(Stress, SS, sizeof Stress);
  if (ct == 30)
    for (int e = 0; e < 9; ++e) SS[e] = X[e] * dt + SS[e];
  else
    for (int e = 0; e < 9; ++e) SS[e] = X[e] * (2.0 * dt) + Sb[e];
  memcpy(Sb, Stress, sizeof Stress);
  if (o->fail[i] == 1) {
    double J2 = J2of(SS);
    double r = o->sigmay[i] / sqrt(3.0 * J2);
    double s = (1.0 < r) ? 1.0 : r; /* std::min(r, 1.0) */
    for (int e = 0; e < 9; ++e) SS[e] = SS[e] * s;
  }
  double* Sig = o->sigma + 9 * i;
  for (int e = 0; e < 9; ++e) Sig[e] = OI[e] * -o->pressure[i] + SS[e];
  double *E = o->strain + 9 * i, *Eb = o->strainb + 9 * i;
  memcpy(Stress, E, sizeof Stress);
  if (ct == 30)
    for (int e = 0; e < 9; ++e) E[e] = SR[e] * dt + E[e];
  else
    for (int e = 0; e < 9; ++e) E[e] = SR[e] * (2.0 * dt) + Eb[e];
  memcpy(Eb, Stress, sizeof Stress);
  if (o->fail[i] > 1) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Undefined failure criteria for solids");
  return PSPH_OK;
}

/* Drucker-Prager constants (Particle.cpp:344-356 / :665-675). */
static void dp_constants(const psph_oracle* o, int64_t i, double* alpha, double* kf) {
  const double phi = o->phi[i], c = o->cohesion[i];
  if (o->I[8] == 0.0) {
    *alpha = tan(phi) / sqrt(9.0 + 12.0 * tan(phi) * tan(phi));
    *kf = 3.0 * c / sqrt(9.0 + 12.0 * tan(phi) * tan(phi));
  } else {
    *alpha = (2.0 * sin(phi)) / (sqrt(3.0) * (3.0 - sin(phi)));
    *kf = (6.0 * c * cos(phi)) / (sqrt(3.0) * (3.0 - sin(phi)));
  }
}

/* Bring a stress back to the apex of the yield cone (Particle.cpp:359-368). */
static double dp_apex(double* S, double alpha, double kf) {
  double I1 = S[0] + S[4] + S[8];
  if ((kf - alpha * I1) < 0.0) {
    double Ratio = (alpha == 0.0) ? 0.0 : kf / alpha;
    S[0] -= 1.0 / 3.0 * (I1 - Ratio);
    S[4] -= 1.0 / 3.0 * (I1 - Ratio);
    S[8] -= 1.0 / 3.0 * (I1 - Ratio);
    I1 = Ratio;
  }
  return I1;
}

static void deviator(const double* S, double I1, double* D) {
  double s = 1.0 / 3.0 * I1;
  for (int e = 0; e < 9; ++e) D[e] = S[e] - OI[e] * s;
}

/* Drucker-Prager plastic corrector + final scale-back, shared by Mat3Leapfrog
 * (Particle.cpp:677-746) and Mat3MVerlet (:357-425). Sig is the elastic
 * predictor (modified in place), Sn the stress at the start of the step,
 * fac the step multiplier of the corrector (dt or 2dt). */
static int dp_return(psph_oracle* o, int64_t i, double* Sig, const double* Sn, const double* SR, double I1strain,
                     double fac) {
  double alpha, kf, SS[9];
  dp_constants(o, i, &alpha, &kf);
  const double K = o->k_mod[i], G = o->g_mod[i];
  double I1 = dp_apex(Sig, alpha, kf);
  deviator(Sig, I1, SS);
  double J2 = J2of(SS);
  if ((sqrt(J2) + alpha * I1 - kf) > 0.0) {
    deviator(Sn, Sn[0] + Sn[4] + Sn[8], SS);
    J2 = J2of(SS);
    if (sqrt(J2) > 0.0) {
      double sum = 0.0, dLanda, Plastic[9];
      for (int e = 0; e < 9; ++e) sum = (e == 0) ? SS[0] * SR[0] : sum + SS[e] * SR[e]; /* abab + sum */
      const double gj = G / sqrt(J2);
      if (o->fail[i] == 2) {
        dLanda = 1.0 / (9.0 * alpha * alpha * K + G) * ((3.0 * alpha * K * I1strain) + (G / sqrt(J2)) * sum);
        double s = 3.0 * alpha * K;
        for (int e = 0; e < 9; ++e) Plastic[e] = o->I[e] * s + SS[e] * gj;
      } else if (o->fail[i] == 3) {
        dLanda = 1.0 / (9.0 * alpha * K * 3.0 * sin(o->psi[i]) + G) * ((3.0 * alpha * K * I1strain) + (G / sqrt(J2)) * sum);
        double s = 3.0 * 3.0 * sin(o->psi[i]) * K;
        for (int e = 0; e < 9; ++e) Plastic[e] = o->I[e] * s + SS[e] * gj;
      } else
        return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Failure Type No is out of range");
      for (int e = 0; e < 9; ++e) Sig[e] = Sig[e] - (Plastic[e] * dLanda) * fac;
    }
    I1 = dp_apex(Sig, alpha, kf);
    deviator(Sig, I1, SS);
    J2 = J2of(SS);
    if ((sqrt(J2) + alpha * I1 - kf) > 0.0 && sqrt(J2) > 0.0) {
      double s1 = I1 / 3.0, s2 = (kf - alpha * I1) / sqrt(J2);
      for (int e = 0; e < 9; ++e) Sig[e] = OI[e] * s1 + SS[e] * s2;
    }
  }
  memcpy(o->shear_stress + 9 * i, SS, sizeof SS); /* Particle::ShearStress keeps the last deviator */
  return PSPH_OK;
}

/* Mat3Leapfrog (Particle.cpp:641-795; porosity update out of scope) */
/* Kozeny-Carman (1), Ergun (2) and Den Adel (3) permeabilities at porosity n
 * (InitialChecks, Source/Domain.cpp:1687-1713; VarPorosity, Particle.cpp:450-474);
 * SeepageType 0 keeps the given k */
static void permeability(psph_oracle* o, int64_t i, double n) {
  const double d = o->d[i];
  switch (o->seepage_type[i]) {
    case 1:
      o->k[i] = n * n * n * d * d / (180.0 * (1.0 - n) * (1.0 - n));
      break;
    case 2:
      o->k[i] = n * n * n * d * d / (150.0 * (1.0 - n) * (1.0 - n));
      o->k2[i] = 1.75 * (1.0 - n) / (n * n * n * d);
      break;
    case 3:
      o->k[i] = n * n * n * d * d / (150.0 * (1.0 - n) * (1.0 - n));
      o->k2[i] = 0.4 / (n * n * d);
      break;
    default:
      break;
  }
}

/* VarPorosity (Source/Particle.cpp:444-479, :757-792): the porosity follows the
 * volumetric strain, n = (n0 + ev) / (1 + ev), and the permeabilities follow n */
static void var_porosity(psph_oracle* o, int64_t i) {
  if (!o->var_porosity[i]) return;
  const double* E = o->strain + 9 * i;
  double ev = (E[0] + E[4] + E[8]);
  permeability(o, i, (o->n0[i] + ev) / (1.0 + ev));
}

static int mat3_leapfrog(psph_oracle* o, int64_t i, double dt) {
  double *Sig = o->sigma + 9 * i, *Sa = o->sigmaa + 9 * i, *Sb = o->sigmab + 9 * i;
  const double *SR = o->strain_rate + 9 * i, *RR = o->rotation_rate + 9 * i;
  double X[9];
  mat3_rate(SR, RR, Sig, o->k_mod[i], o->g_mod[i], X);
  const double I1strain = SR[0] + SR[4] + SR[8];
  if (o->it.first_step)
    for (int e = 0; e < 9; ++e) Sa[e] = X[e] * (-dt / 2.0) + Sig[e];
  for (int e = 0; e < 9; ++e) Sb[e] = Sa[e];
  for (int e = 0; e < 9; ++e) Sa[e] = X[e] * dt + Sa[e];
  if (o->fail[i] > 1) {
    int st = dp_return(o, i, Sa, Sig, SR, I1strain, dt);
    if (st) return st;
  }
  for (int e = 0; e < 9; ++e) Sig[e] = (Sa[e] + Sb[e]) * (1.0 / 2.0);
  double *E = o->strain + 9 * i, *Ea = o->straina + 9 * i, *Eb = o->strainb + 9 * i;
  if (o->it.first_step)
    for (int e = 0; e < 9; ++e) Ea[e] = SR[e] * (-dt / 2.0) + E[e];
  for (int e = 0; e < 9; ++e) Eb[e] = Ea[e];
  for (int e = 0; e < 9; ++e) Ea[e] = SR[e] * dt + Ea[e];
  for (int e = 0; e < 9; ++e) E[e] = (Ea[e] + Eb[e]) * (1.0 / 2.0);
  var_porosity(o, i);
  return PSPH_OK;
}

/* Mat3MVerlet (Particle.cpp:320-482) */
static int mat3_mverlet(psph_oracle* o, int64_t i, double dt, int ct) {
  double *Sig = o->sigma + 9 * i, *Sb = o->sigmab + 9 * i;
  const double *SR = o->strain_rate + 9 * i, *RR = o->rotation_rate + 9 * i;
  double X[9], Stress[9];
  mat3_rate(SR, RR, Sig, o->k_mod[i], o->g_mod[i], X);
  const double I1strain = SR[0] + SR[4] + SR[8];
  memcpy(Stress, Sig, sizeof Stress);
  if (ct == 30)
    for (int e = 0; e < 9; ++e) Sig[e] = X[e] * dt + Sig[e];
  else
    for (int e = 0; e < 9; ++e) Sig[e] = X[e] * (2.0 * dt) + Sb[e];
  memcpy(Sb, Stress, sizeof Stress);
  if (o->fail[i] > 1) {
    int st = dp_return(o, i, Sig, Stress, SR, I1strain, (ct == 30) ? dt : 2.0 * dt);
    if (st) return st;
  }
  double *E = o->strain + 9 * i, *Eb = o->strainb + 9 * i;
  memcpy(Stress, E, sizeof Stress);
  if (ct == 30)
    for (int e = 0; e < 9; ++e) E[e] = SR[e] * dt + E[e];
  else
    for (int e = 0; e < 9; ++e) E[e] = SR[e] * (2.0 * dt) + Eb[e];
  memcpy(Eb, Stress, sizeof Stress);
  var_porosity(o, i);
  return PSPH_OK;
}

/* Domain::Move (Source/Domain.cpp:1299-1325) -> Particle::Move (Particle.cpp:119-144)
 * -> Move_MVerlet (:189-274) | Move_Leapfrog (:561-596). The per-particle
 * counters are advanced once for the domain afterwards. */
static int move(psph_oracle* o, int nthr) {
  const double dt = o->it.deltat;
  const int ct = o->it.ct;
  const int shep_now = (o->it.shepard_counter == o->cfg.shepard_step);
  int status = PSPH_OK;
#pragma omp parallel for schedule(static) num_threads(nthr)
  for (int64_t i = 0; i < o->n; i++) {
    if (!FREE(i)) continue;
    if (o->in_out[i] > 0) {  /* in/out-flow particles keep their prescribed state (Source/Domain.cpp:1305-1320) */
      for (int d = 0; d < 3; ++d) o->a[3 * i + d] = 0.0;
      if (o->in_out[i] == 1 || o->cfg.out_density > 0.0) {
        o->ddensity[i] = 0.0;
        o->zwab[i] = 0.0;
      }
    }
    double* x = o->x + 3 * i;
    double* v = o->v + 3 * i;
    const double* a = o->a + 3 * i;
    if (o->cfg.scheme == PSPH_MVERLET) {
      const double* vx = o->vxsph + 3 * i;
      for (int d = 0; d < 3; ++d) x[d] += dt * (v[d] + vx[d]) + 0.5 * dt * dt * a[d];
      const int shep = o->shepard[i] && shep_now;
      if (ct == 30) {
        if (shep && o->zwab[i] > 0.6) {
          o->densityb[i] = o->sumden[i] / o->zwab[i];
          o->density[i] = o->sumden[i] / o->zwab[i];
        } else {
          o->densityb[i] = o->density[i];
          o->density[i] += dt * o->ddensity[i];
        }
        double* vb = o->vb + 3 * i;
        for (int d = 0; d < 3; ++d) {
          vb[d] = v[d];
          v[d] += dt * a[d];
        }
      } else {
        if (shep && o->zwab[i] > 0.6) {
          o->densityb[i] = o->sumden[i] / o->zwab[i];
          o->density[i] = o->sumden[i] / o->zwab[i];
        } else {
          double dens = o->density[i];
          o->density[i] = o->densityb[i] + 2.0 * dt * o->ddensity[i];
          o->densityb[i] = dens;
        }
        double* vb = o->vb + 3 * i;
        for (int d = 0; d < 3; ++d) {
          double t = v[d];
          v[d] = vb[d] + 2 * dt * a[d];
          vb[d] = t;
        }
      }
      int st = PSPH_OK;
      switch (o->material[i]) {
        case 1: mat1(o, i); break;
        case 2: st = mat2_mverlet(o, i, dt, ct); break;
        default: st = mat3_mverlet(o, i, dt, ct); break;
      }
      if (st) status = st;
    } else {
      double* va = o->va + 3 * i;
      double* vb = o->vb + 3 * i;
      if (o->it.first_step) {
        o->densitya[i] = o->density[i] - dt / 2.0 * o->ddensity[i];
        for (int d = 0; d < 3; ++d) va[d] = v[d] - dt / 2.0 * a[d];
      }
      o->densityb[i] = o->densitya[i];
      o->densitya[i] += dt * o->ddensity[i];
      o->density[i] = (o->densitya[i] + o->densityb[i]) / 2.0;
      for (int d = 0; d < 3; ++d) {
        vb[d] = va[d];
        va[d] += dt * a[d];
        v[d] = (va[d] + vb[d]) / 2.0;
        x[d] += dt * va[d];
      }
      int st = PSPH_OK;
      switch (o->material[i]) {
        case 1: mat1(o, i); break;
        case 2: st = mat2_leapfrog(o, i, dt); break;
        default: st = mat3_leapfrog(o, i, dt); break;
      }
      if (st) status = st;
    }
    /* periodic wrap (Particle.cpp:128-142) */
    for (int d = 0; d < 3; ++d)
      if (o->g.dom_size[d] > 0.0) {
        if (x[d] > o->g.trpr[d]) x[d] -= o->g.dom_size[d];
        if (x[d] < o->g.blpf[d]) x[d] += o->g.dom_size[d];
      }
  }
  if (status) return status;
  if (o->cfg.scheme == PSPH_MVERLET) {
    o->it.ct = (o->it.ct == 30) ? 0 : o->it.ct + 1;
    o->it.shepard_counter = (o->it.shepard_counter == o->cfg.shepard_step) ? 0 : o->it.shepard_counter + 1;
  }
  o->it.first_step = 0;
  return PSPH_OK;
}

/* CheckParticleLeave (Source/Domain.cpp:517-547): order-preserving removal. */
static void check_particle_leave(psph_oracle* o) {
  int64_t k = 0;
  for (int64_t i = 0; i < o->n; ++i) {
    const double* x = o->x + 3 * i;
    int out = 0;
    for (int d = 0; d < 3; ++d) out |= (x[d] > o->g.trpr[d]) || (x[d] < o->g.blpf[d]);
    if (out) continue;
    if (k != i) {
#define MOVE_I(NAME) o->NAME[k] = o->NAME[i];
#define MOVE_D(NAME) o->NAME[k] = o->NAME[i];
#define MOVE_V(NAME) memmove(o->NAME + 3 * k, o->NAME + 3 * i, 3 * sizeof(double));
#define MOVE_T(NAME) memmove(o->NAME + 9 * k, o->NAME + 9 * i, 9 * sizeof(double));
      PSPH_INT_FIELDS(MOVE_I)
      PSPH_F64_FIELDS(MOVE_D)
      PSPH_VEC_FIELDS(MOVE_V)
      PSPH_TEN_FIELDS(MOVE_T)
      o->orig[k] = o->orig[i];
    }
    k++;
  }
  o->n = k;
}

/* Grows every per-particle array to hold n_new particles (appended ones start
 * zeroed; the caller fills them as the Particle constructor would). */
static void grow(psph_oracle* o, int64_t n_new) {
  const int64_t n = o->n;
#define GROW_I(NAME) o->NAME = (int32_t*)realloc(o->NAME, (size_t)n_new * sizeof(int32_t)); memset(o->NAME + n, 0, (size_t)(n_new - n) * sizeof(int32_t));
#define GROW_D(NAME) o->NAME = (double*)realloc(o->NAME, (size_t)n_new * sizeof(double)); memset(o->NAME + n, 0, (size_t)(n_new - n) * sizeof(double));
#define GROW_V(NAME) o->NAME = (double*)realloc(o->NAME, (size_t)n_new * 3 * sizeof(double)); memset(o->NAME + 3 * n, 0, (size_t)(n_new - n) * 3 * sizeof(double));
#define GROW_T(NAME) o->NAME = (double*)realloc(o->NAME, (size_t)n_new * 9 * sizeof(double)); memset(o->NAME + 9 * n, 0, (size_t)(n_new - n) * 9 * sizeof(double));
  PSPH_INT_FIELDS(GROW_I)
  PSPH_F64_FIELDS(GROW_D)
  PSPH_VEC_FIELDS(GROW_V)
  PSPH_TEN_FIELDS(GROW_T)
  o->orig = (int64_t*)realloc(o->orig, (size_t)n_new * sizeof(int64_t));
  o->LL = (int32_t*)realloc(o->LL, (size_t)n_new * sizeof(int32_t));
  o->CC = (int32_t*)realloc(o->CC, (size_t)n_new * 3 * sizeof(int32_t));
  o->fixed = (int64_t*)realloc(o->fixed, (size_t)n_new * sizeof(int64_t));
  o->a_scale = (double*)realloc(o->a_scale, (size_t)n_new * sizeof(double));
  o->dr_scale = (double*)realloc(o->dr_scale, (size_t)n_new * sizeof(double));
  o->satcheck = (int32_t*)realloc(o->satcheck, (size_t)n_new * sizeof(int32_t));
  o->fsi_p = (double*)realloc(o->fsi_p, (size_t)n_new * sizeof(double));
  o->fsi_sk = (double*)realloc(o->fsi_sk, (size_t)n_new * sizeof(double));
  o->fsi_cnt = (int32_t*)realloc(o->fsi_cnt, (size_t)n_new * sizeof(int32_t));
  o->fsi_nsv = (double*)realloc(o->fsi_nsv, (size_t)n_new * 3 * sizeof(double));
  o->locks = (omp_lock_t*)realloc(o->locks, (size_t)n_new * sizeof(omp_lock_t));
  for (int64_t i = n; i < n_new; ++i) {
    omp_init_lock(&o->locks[i]);
    o->orig[i] = o->next_orig++;
    o->LL[i] = -1;
  }
  o->n = n_new;
}

static void in_part_push(psph_oracle* o, int64_t a) {
  if (o->n_in_part == o->cap_in_part) {
    o->cap_in_part = o->cap_in_part ? 2 * o->cap_in_part : 256;
    o->in_part = (int64_t*)realloc(o->in_part, (size_t)o->cap_in_part * sizeof(int64_t));
  }
  o->in_part[o->n_in_part++] = a;
}

/* The particles of the cells with x index in [qa, qb) in InFlowBCFresh's
 * traversal order (q2, q3, q1, then each cell's chain), for which keep()
 * holds (Source/Domain.cpp:1508-1530). */
#define FLOW_TRAVERSE(o, qa, qb, BODY)                                                        \
  for (int q2 = 0; o->cfg.periodic[1] ? (q2 < (o->g.cell_no[1] - 2)) : (q2 < o->g.cell_no[1]); q2++) \
    for (int q3 = 0; o->cfg.periodic[2] ? (q3 < (o->g.cell_no[2] - 2)) : (q3 < o->g.cell_no[2]); q3++) \
      for (int q1 = (qa); q1 < (qb); q1++) {                                                   \
        int32_t temp = HOCI(o, q1, q2, q3);                                                    \
        while (temp != -1) {                                                                   \
          BODY;                                                                                \
          temp = o->LL[temp];                                                                  \
        }                                                                                      \
      }

/* InCon / OutCon: the reference's default hooks, InFlowCon and OutFlowCon
 * (Source/Domain.cpp:35-45), give BC.inv / inDensity and BC.outv / outDensity */
static void set_flow_state(psph_oracle* o, int64_t a, const double* vel, double den, int set_v, int set_d) {
  if (set_v)
    for (int d = 0; d < 3; ++d) o->v[3 * a + d] = o->vb[3 * a + d] = o->va[3 * a + d] = vel[d];
  if (set_d) {
    o->density[a] = o->densityb[a] = o->densitya[a] = den;
    o->pressure[a] = EOS(o->pres_eq[a], o->cs[a], o->p0[a], o->density[a], o->ref_density[a]);
  }
}

/* InFlowBCFresh (Source/Domain.cpp:1490-1636) */
static int in_flow_fresh(psph_oracle* o) {
  const psph_config* c = &o->cfg;
  const double cellfac = c->bc_cellfac > 0.0 ? c->bc_cellfac : 3.9;
  const int iof = c->in_out_flow;
  if (o->inoutcounter == 0) {
    if (iof == 1 || iof == 3) {
      const double* inv = c->in_v;
      if (!(sqrt(dot3(inv, inv)) > 0.0) || !(c->in_density > 0.0))
        return fail(o, PSPH_ERR_INVALID_ARGUMENT, "BC.inv or BC.inDensity are not defined");
      o->n_in_part = 0;
      o->in_loc1 = o->g.blpf[0] + cellfac * o->g.hmax;
      const int temp1 = (int)(floor((o->in_loc1 - o->g.blpf[0]) / o->g.cell_size[0]));
      FLOW_TRAVERSE(o, 0, temp1 + 1, if (FREE(temp) && (o->x[3 * temp] <= o->in_loc1)) {
        in_part_push(o, temp);
        o->in_out[temp] = 1;
      })
      if (o->n_in_part == 0) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "no free particle in the in-flow zone");
      o->in_loc2 = o->in_loc3 = o->x[3 * o->in_part[0]];
      for (int64_t i = 0; i < o->n_in_part; i++) {
        const double x0 = o->x[3 * o->in_part[i]];
        if (x0 < o->in_loc2) o->in_loc2 = x0;
        if (x0 > o->in_loc3) o->in_loc3 = x0;
      }
    }
    if (iof == 2 || iof == 3) o->out_loc = o->g.trpr[0] - cellfac * o->g.hmax;
    o->inoutcounter = 2;
  }
  if (o->inoutcounter == 1) {
    o->n_in_part = 0;
    const int temp1 = (int)(floor((o->in_loc1 - o->g.blpf[0]) / o->g.cell_size[0]));
    FLOW_TRAVERSE(o, 0, temp1 + 1, if (FREE(temp) && (o->x[3 * temp] <= o->in_loc1) && o->in_out[temp] == 1)
                                       in_part_push(o, temp))
    o->inoutcounter = 2;
  }
  o->n_out_part = 0;
  if (iof == 2 || iof == 3) {
    const int temp1 = (int)(floor((o->out_loc - o->g.blpf[0]) / o->g.cell_size[0]));
    FLOW_TRAVERSE(o, temp1, o->g.cell_no[0], if (FREE(temp) && (o->x[3 * temp] >= o->out_loc)) {
      o->in_out[temp] = 2;
      o->n_out_part++;
    })
  }
  /* InCon on BC.InPart, in list order (Source/Domain.cpp:1594-1608) */
  for (int64_t i = 0; i < o->n_in_part; i++) {
    const int64_t a = o->in_part[i];
    if (o->flow_fn[PSPH_FLOW_IN]) {
      double vel[3] = {0.0, 0.0, 0.0}, den = 0.0;
      o->flow_fn[PSPH_FLOW_IN](&o->x[3 * a], vel, &den, o->flow_user[PSPH_FLOW_IN]);
      set_flow_state(o, a, vel, den, 1, 1);
    } else {
      set_flow_state(o, a, c->in_v, c->in_density, 1, 1);
    }
  }
  /* OutCon on BC.OutPart (Source/Domain.cpp:1610-1633) */
  const double temp11 = c->mass_conservation ? o->n_in_part * 1.0 / (o->n_out_part * 1.0) : 1.0;
  if (o->n_out_part > 0) {
    const int set_v = sqrt(dot3(c->out_v, c->out_v)) > 0.0 || temp11 != 1.0;
    for (int64_t a = 0; a < o->n; a++)
      if (o->in_out[a] == 2 && FREE(a) && o->x[3 * a] >= o->out_loc) {
        double vel[3], den = c->out_density;
        if (o->flow_fn[PSPH_FLOW_OUT]) {
          double hv[3] = {0.0, 0.0, 0.0};
          den = 0.0;
          o->flow_fn[PSPH_FLOW_OUT](&o->x[3 * a], hv, &den, o->flow_user[PSPH_FLOW_OUT]);
          for (int d = 0; d < 3; ++d) vel[d] = temp11 * hv[d];
        } else {
          for (int d = 0; d < 3; ++d) vel[d] = temp11 * c->out_v[d];
        }
        set_flow_state(o, a, vel, den, set_v, c->out_density > 0.0);
      }
  }
  return PSPH_OK;
}

/* The fields InFlowBCLeave copies from in-flow particle b into the recycled
 * particle a (Source/Domain.cpp:1363-1395). */
static void recycle_from(psph_oracle* o, int64_t a, int64_t b, const double* pos) {
  for (int d = 0; d < 3; ++d) o->x[3 * a + d] = pos[d];
  o->material[a] = 1;
  o->in_out[a] = 1;
  o->p0[a] = o->p0[b];
  o->pres_eq[a] = o->pres_eq[b];
  o->cs[a] = o->cs[b];
  o->alpha[a] = o->alpha[b];
  o->beta[a] = o->beta[b];
  o->mu[a] = o->mu[b];
  o->mu_ref[a] = o->mu_ref[b];
  o->t0[a] = 0.0;
  o->mass[a] = o->mass[b];
  o->h[a] = o->h[b];
  o->id[a] = o->id[b];
  o->ti[a] = 0.0;
  o->ref_density[a] = o->ref_density[b];
  o->shepard[a] = o->shepard[b];
  o->les[a] = o->les[b];
  o->csmag[a] = o->csmag[b];
}

/* InFlowBCLeave (Source/Domain.cpp:1327-1488), replacing CheckParticleLeave:
 * particles outside the grid box free their slots (DelPart, index order);
 * in-flow particles that crossed InFlowLoc1 leave the in-flow state and a
 * copy of each, shifted back by the in-flow zone's width, takes a freed slot
 * or is appended (AddPart, InPart order); unused slots are deleted. */
static void in_flow_leave(psph_oracle* o) {
  const psph_config* c = &o->cfg;
  int64_t *del = (int64_t*)malloc((size_t)(o->n ? o->n : 1) * sizeof(int64_t)), ndel = 0;
  for (int64_t i = 0; i < o->n; i++) {
    const double* x = o->x + 3 * i;
    if ((x[0] > o->g.trpr[0]) || (x[1] > o->g.trpr[1]) || (x[2] > o->g.trpr[2]) || (x[0] < o->g.blpf[0]) ||
        (x[1] < o->g.blpf[1]) || (x[2] < o->g.blpf[2])) {
      o->in_out[i] = 0;
      del[ndel++] = i;
    }
  }
  int64_t nadd = 0;
  int64_t* add_b = (int64_t*)malloc((size_t)(o->n_in_part ? o->n_in_part : 1) * sizeof(int64_t));
  double* add_x = (double*)malloc((size_t)(o->n_in_part ? o->n_in_part : 1) * 3 * sizeof(double));
  if (c->in_out_flow == 1 || c->in_out_flow == 3) {
    int64_t keep = 0;
    for (int64_t i = 0; i < o->n_in_part; i++) {
      const int64_t b = o->in_part[i];
      if (o->x[3 * b] > o->in_loc1) {
        for (int d = 0; d < 3; ++d) add_x[3 * nadd + d] = o->x[3 * b + d];
        add_x[3 * nadd] -= (o->in_loc3 - o->in_loc2 + c->initial_dist);
        o->in_out[b] = 0;
        add_b[nadd++] = b;
      } else {
        o->in_part[keep++] = b;
      }
    }
    o->n_in_part = keep;
  }
  if (nadd >= ndel) {
    for (int64_t i = 0; i < ndel; i++) {
      recycle_from(o, del[i], add_b[i], add_x + 3 * i);
      in_part_push(o, del[i]);
    }
    if (nadd != ndel) {
      const int64_t n0 = o->n;
      grow(o, n0 + (nadd - ndel));
      for (int64_t i = ndel; i < nadd; i++) {
        const int64_t a = n0 + (i - ndel), b = add_b[i];
        /* new Particle(ID_b, x, v_b, Mass_b, RefDensity_b, h_b, false): constructor defaults */
        o->is_free[a] = 1;
        o->fpmassc[a] = 1.0;
        o->bingham_m[a] = 300.0;
        o->csmag[a] = 0.17;
        o->tin[a] = 4.0;
        for (int d = 0; d < 3; ++d) o->v[3 * a + d] = o->v[3 * b + d];
        o->density[a] = o->ref_density[b];
        o->volume[a] = o->mass[b] / o->ref_density[b];
        recycle_from(o, a, b, add_x + 3 * i);
        in_part_push(o, a);
      }
    }
  } else {
    for (int64_t i = 0; i < nadd; i++) {
      recycle_from(o, del[i], add_b[i], add_x + 3 * i);
      in_part_push(o, del[i]);
    }
    /* DelItems of the unused slots; InPart holds indices and is rebuilt next step */
    int64_t k = 0, next = nadd;
    for (int64_t i = 0; i < o->n; ++i) {
      if (next < ndel && del[next] == i) {
        next++;
        continue;
      }
      if (k != i) {
#define MOVE_I2(NAME) o->NAME[k] = o->NAME[i];
#define MOVE_D2(NAME) o->NAME[k] = o->NAME[i];
#define MOVE_V2(NAME) memmove(o->NAME + 3 * k, o->NAME + 3 * i, 3 * sizeof(double));
#define MOVE_T2(NAME) memmove(o->NAME + 9 * k, o->NAME + 9 * i, 9 * sizeof(double));
        PSPH_INT_FIELDS(MOVE_I2)
        PSPH_F64_FIELDS(MOVE_D2)
        PSPH_VEC_FIELDS(MOVE_V2)
        PSPH_TEN_FIELDS(MOVE_T2)
        o->orig[k] = o->orig[i];
      }
      k++;
    }
    o->n = k;
    o->inoutcounter = 1;
  }
  free(del);
  free(add_b);
  free(add_x);
}

static int one_step(psph_oracle* o, int nthr) {
  double t0 = now_s();
  start_acceleration(o, nthr);
  if (o->cfg.in_out_flow > 0) {
    int st = in_flow_fresh(o);
    if (st) return st;
  }
  /* FirstStep of Move_MVerlet forces ct=30 (Particle.cpp:191-195) */
  if (o->cfg.scheme == PSPH_MVERLET && o->it.first_step) o->it.ct = 30;
  main_search(o, nthr);
  /* GeneralBefore (Source/Domain.cpp:1767) */
  if (o->hook_fn && (o->hook_mask & PSPH_HOOK_BEFORE) && o->hook_fn(o, PSPH_HOOK_BEFORE, o->hook_user))
    return fail(o, PSPH_ERR_STATE, "the GeneralBefore hook asked to stop the run");
  double t1 = now_s();
  primary_compute(o, nthr);
  double t2 = now_s();
  int st = last_compute(o, nthr);
  if (st) return st;
  /* GeneralAfter (Source/Domain.cpp:1770) */
  if (o->hook_fn && (o->hook_mask & PSPH_HOOK_AFTER) && o->hook_fn(o, PSPH_HOOK_AFTER, o->hook_user))
    return fail(o, PSPH_ERR_STATE, "the GeneralAfter hook asked to stop the run");
  double t3 = now_s();
  st = adaptive_time_step(o);
  if (st) return st;
  st = move(o, nthr);
  if (st) return st;
  o->it.time += o->it.deltat;
  o->it.steps += 1;
  double t4 = now_s();
  if (o->cfg.in_out_flow > 0) in_flow_leave(o);
  else check_particle_leave(o);
  cell_reset(o);
  st = list_generate(o);
  double t5 = now_s();
  o->phase_s[0] += t1 - t0;
  o->phase_s[1] += t2 - t1;
  o->phase_s[2] += t3 - t2;
  o->phase_s[3] += t4 - t3;
  o->phase_s[4] += t5 - t4;
  return st;
}

/* ---------------------------------------------------------------------------
 * Public entry points
 * ------------------------------------------------------------------------- */

static int validate(psph_oracle* o) {
  const psph_config* c = &o->cfg;
  if (c->dimension != 2 && c->dimension != 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Please correct the dimension (2=>2D or 3=>3D)");
  if (c->kernel_type < 0 || c->kernel_type > 2) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Kernel Type No is out of range");
  if (c->vis_eq < 0 || c->vis_eq > 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Viscosity Equation No is out of range");
  if (c->swi_type < 0 || c->swi_type > 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Soil-Water Interaction Type No is out of range");
  if (c->in_out_flow < 0 || c->in_out_flow > 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "InOutFlow is out of range");
  if (c->in_out_flow > 0 && c->periodic[0])
    return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Periodic BC in the X direction cannot be used with In/Out-Flow BC simultaneously");
  for (int64_t i = 0; i < o->n && c->in_out_flow > 0; ++i)
    if (o->shepard[i])
      return fail(o, PSPH_ERR_UNSUPPORTED, "Shepard filtering with in/out-flow (the released particles' own Shepard counters)");
  for (int64_t i = 0; i < o->n; ++i) {
    if (o->material[i] < 1 || o->material[i] > 3) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Material Type No is out of range");
    if (o->pres_eq[i] < 0 || o->pres_eq[i] > 2) return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Please correct Pressure Equation No");
    if (o->material[i] == 3 && (o->seepage_type[i] < 0 || o->seepage_type[i] > 3))
      return fail(o, PSPH_ERR_INVALID_ARGUMENT, "Seepage Type No is out of range");
  }
  return PSPH_OK;
}

psph_oracle* psph_oracle_create(const psph_config* cfg, const psph_particles* p, int initial, const psph_grid* grid,
                                const psph_integrator* integ) {
  psph_oracle* o = (psph_oracle*)calloc(1, sizeof(psph_oracle));
  o->cfg = *cfg;
  const int64_t n = p->n;
  o->n = n;
#define ALLOC_I(NAME) o->NAME = (int32_t*)calloc((size_t)(n ? n : 1), sizeof(int32_t));
#define ALLOC_D(NAME) o->NAME = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
#define ALLOC_V(NAME) o->NAME = (double*)calloc((size_t)(n ? n : 1) * 3, sizeof(double));
#define ALLOC_T(NAME) o->NAME = (double*)calloc((size_t)(n ? n : 1) * 9, sizeof(double));
  PSPH_INT_FIELDS(ALLOC_I)
  PSPH_F64_FIELDS(ALLOC_D)
  PSPH_VEC_FIELDS(ALLOC_V)
  PSPH_TEN_FIELDS(ALLOC_T)
  /* Particle constructor defaults (Source/Particle.cpp:25-117) */
  for (int64_t i = 0; i < n; ++i) {
    o->is_free[i] = 1;
    o->fpmassc[i] = 1.0;
    o->bingham_m[i] = 300.0;
    o->csmag[i] = 0.17;
    o->tin[i] = 4.0;
  }
#define COPY_I(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * sizeof(int32_t));
#define COPY_D(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * sizeof(double));
#define COPY_V(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * 3 * sizeof(double));
#define COPY_T(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * 9 * sizeof(double));
  PSPH_INT_FIELDS(COPY_I)
  PSPH_F64_FIELDS(COPY_D)
  PSPH_VEC_FIELDS(COPY_V)
  PSPH_TEN_FIELDS(COPY_T)
  if (!p->ref_density && p->density) memcpy(o->ref_density, p->density, (size_t)n * sizeof(double));
  /* Particle::V = Mass / RefDensity (the constructor's value, Source/Particle.cpp:88) */
  if (!p->volume)
    for (int64_t i = 0; i < n; ++i) o->volume[i] = o->mass[i] / o->ref_density[i];
  o->satcheck = (int32_t*)calloc((size_t)(n ? n : 1), sizeof(int32_t));
  o->fsi_p = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
  o->fsi_sk = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
  o->fsi_nsv = (double*)calloc((size_t)(n ? n : 1) * 3, sizeof(double));
  o->fsi_cnt = (int32_t*)calloc((size_t)(n ? n : 1), sizeof(int32_t));
  o->orig = (int64_t*)malloc((size_t)(n ? n : 1) * sizeof(int64_t));
  for (int64_t i = 0; i < n; ++i) o->orig[i] = i;
  o->next_orig = n;
  o->LL = (int32_t*)malloc((size_t)(n ? n : 1) * sizeof(int32_t));
  o->CC = (int32_t*)calloc((size_t)(n ? n : 1) * 3, sizeof(int32_t));
  o->fixed = (int64_t*)malloc((size_t)(n ? n : 1) * sizeof(int64_t));
  o->a_scale = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
  o->dr_scale = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
  o->locks = (omp_lock_t*)malloc((size_t)(n ? n : 1) * sizeof(omp_lock_t));
  for (int64_t i = 0; i < n; ++i) omp_init_lock(&o->locks[i]);
  o->nthr = omp_get_max_threads() > 0 ? omp_get_max_threads() : 1;
  if (o->nthr < 256) o->nthr = 256;
  o->sm = (pairvec*)calloc(o->nthr, sizeof(pairvec));
  o->fsm = (pairvec*)calloc(o->nthr, sizeof(pairvec));
  o->nsm = (pairvec*)calloc(o->nthr, sizeof(pairvec));
  for (int e = 0; e < 9; ++e) o->I[e] = OI[e];
  if (cfg->dimension == 2) o->I[8] = 0.0;
  o->g.cellfac = (cfg->kernel_type == 2) ? 3.0 : 2.0; /* Kernel_Set (Source/Domain.cpp:117-121) */
  o->it.time = cfg->time;
  o->it.deltat = o->it.deltatint = o->it.deltatmin = cfg->dt;
  o->it.first_step = 1;
  if (validate(o)) return o;
  if (integ) o->it = *integ;
  if (initial) {
    /* InitialChecks (Source/Domain.cpp:1662-1678): initial EOS pressure */
    for (int64_t i = 0; i < n; i++)
      if (o->material[i] < 3) o->pressure[i] = EOS(o->pres_eq[i], o->cs[i], o->p0[i], o->density[i], o->ref_density[i]);
    /* permeabilities of the soil from its porosity (Source/Domain.cpp:1680-1716) */
    for (int64_t i = 0; i < n; i++)
      if (o->material[i] == 3) permeability(o, i, o->n0[i]);
  }
  if (grid) {
    o->g = *grid;
  } else if (cell_initiate(o)) {
    return o;
  }
  if (alloc_cells(o)) return o;
  if (list_generate(o)) return o;
  if (initial && !grid) {
    /* TimestepCheck (Source/Domain.cpp:1721-1733) */
    double t1 = 0.25 * o->g.hmax / (o->cs_max), t2;
    if (o->mu_max > 0.0) t2 = 0.125 * o->g.hmax * o->g.hmax * o->g.rhomax / o->mu_max; else t2 = 1000000.0;
    if (o->it.deltatint > (t1 < t2 ? t1 : t2)) fail(o, PSPH_ERR_CFL, "Please decrease the time step to the allowable range");
  }
  return o;
}

void psph_oracle_destroy(psph_oracle* o) {
  if (!o) return;
#define FREE_F(NAME) free(o->NAME);
  PSPH_INT_FIELDS(FREE_F)
  PSPH_F64_FIELDS(FREE_F)
  PSPH_VEC_FIELDS(FREE_F)
  PSPH_TEN_FIELDS(FREE_F)
  for (int64_t i = 0; i < o->n; ++i) omp_destroy_lock(&o->locks[i]);
  for (int t = 0; t < o->nthr; ++t) {
    free(o->sm[t].v);
    free(o->fsm[t].v);
    free(o->nsm[t].v);
  }
  free(o->sm);
  free(o->fsm);
  free(o->nsm);
  free(o->orig);
  free(o->LL);
  free(o->CC);
  free(o->HOC);
  free(o->satcheck);
  free(o->fsi_p);
  free(o->fsi_sk);
  free(o->fsi_nsv);
  free(o->fsi_cnt);
  free(o->in_part);
  free(o->fixed);
  free(o->a_scale);
  free(o->dr_scale);
  free(o->locks);
  free(o);
}

const char* psph_oracle_error(const psph_oracle* o) { return o->status ? o->err : ""; }

int psph_oracle_step(psph_oracle* o, int64_t nsteps, int nthreads) {
  if (o->status) return o->status;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > o->nthr) nthreads = o->nthr;
  for (int e = 0; e < 5; ++e) o->phase_s[e] = 0.0;
  for (int64_t s = 0; s < nsteps; ++s) {
    int st = one_step(o, nthreads);
    if (st) return fail(o, st, "%s", o->err[0] ? o->err : "step failed");
  }
  return PSPH_OK;
}

int64_t psph_oracle_num_particles(const psph_oracle* o) { return o->n; }

int psph_oracle_download(const psph_oracle* o, psph_particles* out) {
  const int64_t n = o->n;
  if (out->n < n) return PSPH_ERR_INVALID_ARGUMENT;
#define OUT_I(NAME) if (out->NAME) memcpy(out->NAME, o->NAME, (size_t)n * sizeof(int32_t));
#define OUT_D(NAME) if (out->NAME) memcpy(out->NAME, o->NAME, (size_t)n * sizeof(double));
#define OUT_V(NAME) if (out->NAME) memcpy(out->NAME, o->NAME, (size_t)n * 3 * sizeof(double));
#define OUT_T(NAME) if (out->NAME) memcpy(out->NAME, o->NAME, (size_t)n * 9 * sizeof(double));
  PSPH_INT_FIELDS(OUT_I)
  PSPH_F64_FIELDS(OUT_D)
  PSPH_VEC_FIELDS(OUT_V)
  PSPH_TEN_FIELDS(OUT_T)
  return PSPH_OK;
}

int psph_oracle_original_index(const psph_oracle* o, int64_t* out) {
  memcpy(out, o->orig, (size_t)o->n * sizeof(int64_t));
  return PSPH_OK;
}

int psph_oracle_get_grid(const psph_oracle* o, psph_grid* g) {
  *g = o->g;
  return PSPH_OK;
}

int psph_oracle_get_integrator(const psph_oracle* o, psph_integrator* it) {
  *it = o->it;
  return PSPH_OK;
}

int64_t psph_oracle_pairs(psph_oracle* o, int which, int64_t* buf, int64_t cap) {
  if (o->status) return -1;
  main_search(o, 1);
  int64_t cnt = 0;
  for (int k = 0; k < o->nthr; ++k) {
    pairvec* lists[3] = {&o->sm[k], &o->fsm[k], &o->nsm[k]};
    for (int l = 0; l < 3; ++l) {
      if (which < 3 && l != which) continue;
      for (int64_t i = 0; i < lists[l]->n; ++i) {
        int64_t p1 = lists[l]->v[2 * i], p2 = lists[l]->v[2 * i + 1];
        if (which == 3) {
          double xij[3];
          for (int d = 0; d < 3; ++d) xij[d] = o->x[3 * p1 + d] - o->x[3 * p2 + d];
          double h = (o->h[p1] + o->h[p2]) / 2;
          periodic_correction(o, xij, h, p1, p2);
          if (sqrt(dot3(xij, xij)) / h > o->g.cellfac) continue;
        }
        if (cnt < cap) {
          buf[2 * cnt] = o->orig[p1];
          buf[2 * cnt + 1] = o->orig[p2];
        }
        cnt++;
      }
    }
  }
  for (int t = 0; t < o->nthr; ++t) o->sm[t].n = o->fsm[t].n = o->nsm[t].n = 0;
  return cnt;
}

int psph_oracle_scales(const psph_oracle* o, double* a_scale, double* drho_scale) {
  memcpy(a_scale, o->a_scale, (size_t)o->n * sizeof(double));
  memcpy(drho_scale, o->dr_scale, (size_t)o->n * sizeof(double));
  return PSPH_OK;
}

int64_t psph_oracle_pair_count(const psph_oracle* o) { return o->pairs_done; }

int psph_oracle_phase_times(const psph_oracle* o, double* s, int cap) {
  for (int e = 0; e < 5 && e < cap; ++e) s[e] = o->phase_s[e];
  return 5;
}

int psph_oracle_set_flow_profile(psph_oracle* o, int which, psph_flow_fn fn, void* user) {
  if (!o || (which != PSPH_FLOW_IN && which != PSPH_FLOW_OUT)) return PSPH_ERR_INVALID_ARGUMENT;
  o->flow_fn[which] = fn;
  o->flow_user[which] = fn ? user : NULL;
  return PSPH_OK;
}

int psph_oracle_set_step_hooks(psph_oracle* o, psph_oracle_hook_fn fn, void* user, int where_mask) {
  if (!o) return PSPH_ERR_INVALID_ARGUMENT;
  o->hook_fn = fn;
  o->hook_user = fn ? user : NULL;
  o->hook_mask = fn ? where_mask : 0;
  return PSPH_OK;
}

/* The non-NULL arrays of p (psph_oracle_download's order and count) replace
 * the particles' fields; k, k2 and the in/out-flow flags are left, as
 * psph_patch leaves them. */
int psph_oracle_patch(psph_oracle* o, const psph_particles* p) {
  if (!o || !p || p->n != o->n) return PSPH_ERR_INVALID_ARGUMENT;
  const int64_t n = o->n;
#define IN_I(NAME) if (p->NAME && strcmp(#NAME, "in_out") != 0) memcpy(o->NAME, p->NAME, (size_t)n * sizeof(int32_t));
#define IN_D(NAME) if (p->NAME && strcmp(#NAME, "k") != 0 && strcmp(#NAME, "k2") != 0) memcpy(o->NAME, p->NAME, (size_t)n * sizeof(double));
#define IN_V(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * 3 * sizeof(double));
#define IN_T(NAME) if (p->NAME) memcpy(o->NAME, p->NAME, (size_t)n * 9 * sizeof(double));
  PSPH_INT_FIELDS(IN_I)
  PSPH_F64_FIELDS(IN_D)
  PSPH_VEC_FIELDS(IN_V)
  PSPH_TEN_FIELDS(IN_T)
  return PSPH_OK;
}
