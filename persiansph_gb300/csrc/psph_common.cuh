// Shared device-side definitions for the GB300 hot path.
//
// Device data layout (structure of arrays, sorted by cell every step):
//   X4[s]  = (x, y, z, Density)            persistent, reordered
//   V4[s]  = (vx, vy, vz, Pressure)        persistent, reordered
//   H4[s]  = (va|vb xyz, Densitya|Densityb) persistent, reordered (scheme's history)
//   cls[s] = particle-class index           persistent, reordered
//   orig[s]= original particle index        persistent, reordered
// Per-particle constants (material, flags, EOS, viscosity, soil parameters,
// mass, h) are de-duplicated on upload into a small class table (PClass).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "psph.h"

#define PSPH_HD __host__ __device__ __forceinline__
#define PSPH_D __device__ __forceinline__

namespace psph {

constexpr double kPi = 3.14159265358979323846;

// Status bits raised by kernels (read back by the host after each call).
enum : uint32_t {
  ST_NONFINITE = 1u << 0,
  ST_DT_COLLAPSE = 1u << 1,
  ST_OUT_OF_GRID = 1u << 2,
  ST_CELL_OVERFLOW = 1u << 3,
  ST_CLOSURE_TIMEOUT = 1u << 4,  // a tensor-core wait of the closure kernel gave up
  ST_STAGE_TIMEOUT = 1u << 5,    // a shared-memory staging wait of the neighbour scan gave up
  ST_LIST_MISMATCH = 1u << 6,    // a pair inside the support missing from its partner's list
};

// Constant per-particle parameters, shared by all particles of one class.
struct PClass {
  double cs, p0, rho0, fpmassc, alpha, beta, mu0, mu_ref, t0, bm, csmag, ti, tin, tid;
  double g_mod, k_mod, sigmay, coh, phi, psi, h, mass;
  // soil-water interaction of soil classes (Source/Particle.h:110-121): initial
  // porosity, permeabilities k and k2 (InitialChecks' values), grain size d,
  // fluid density RhoF, particle volume V
  double n0, kp, kp2, dgrain, rho_f, vol;
  // Drucker-Prager constants of the class (alpha, k_f, sin psi), derived on the
  // device once after upload with the same expressions the return mapping
  // used per particle (zero while the table is built on the host)
  double dp_alpha, dp_kf, dp_sin_psi;
  // Tait EOS constants of the class for the FP32C update (class_constants_kernel):
  // B = rho0 cs^2 / 7 (the reference's expression), 1/rho0, B in FP32
  double eos_b, eos_inv_rho0;
  float eos_b32;
  int material, is_free, no_slip, pres_eq, shepard, les, vis_m, fail, id, inst;
  int seep_type, var_por, is_sat;
  // the class a particle of this class moves to when its saturation changes
  // (saturated soil weighs its buoyant weight); set after the table is built
  int twin;
};

// FP32 copy of the class constants used inside the FP32C pair loops (so those
// loops issue no FP64 instructions), with the boolean switches as bits.
struct PClass32 {
  float mass, h, fpmassc, alpha, beta, mu0, ti, tin, tid, cs, rho0, p0;
  float h_over_dx;  // closure feature h / dx, rounded from FP64 as the FP64 form does (set at attach)
  int flags;  // bit 0 free, 1 no-slip, 2 LES, 3 Shepard, 4 T0>0, 5 TI>0
  int material, pres_eq, inst;
};
enum : int { CF_FREE = 1, CF_NOSLIP = 2, CF_LES = 4, CF_SHEPARD = 8, CF_T0 = 16, CF_TI = 32 };

// Kozeny-Carman (1), Ergun (2) and Den Adel (3) permeabilities of soil at
// porosity n and grain size d, in the reference's expression order
// (InitialChecks, Source/Domain.cpp:1687-1713; VarPorosity, Source/Particle.cpp:450-474);
// SeepageType 0 keeps the given k and k2.
PSPH_HD void permeability(int type, double n, double d, double* k, double* k2) {
  if (type == 1) {
    *k = n * n * n * d * d / (180.0 * (1.0 - n) * (1.0 - n));
  } else if (type == 2) {
    *k = n * n * n * d * d / (150.0 * (1.0 - n) * (1.0 - n));
    *k2 = 1.75 * (1.0 - n) / (n * n * n * d);
  } else if (type == 3) {
    *k = n * n * n * d * d / (150.0 * (1.0 - n) * (1.0 - n));
    *k2 = 0.4 / (n * n * d);
  }
}

// Per-instance (per-domain) scalars advanced on the device. A context holds one
// instance for a single Domain, or many independent instances for an ensemble.
struct InstState {
  double time, deltat, deltatint, deltatmin, t_stop;
  long long steps;
  unsigned long long dtmin_bits;  // running minimum of the acceleration time-step bound (ordered bits)
  int first_step, ct, shepard_counter, stop;
  int k_initial;  // the first step after an initial upload: permeabilities are InitialChecks' values
  int pad;
};

// Context-wide scalars.
struct StepScalars {
  int n;          // particles alive (cells + orphans), all instances
  int n_cells;    // particles inside cells
  int n_total;
  uint32_t status;
  int all_stop;   // every instance has reached its stop time
  int buf;        // which persistent buffer (A=0 / B=1) holds the current sorted state
  unsigned long long pairs_x2;  // 2 x pair-interactions evaluated since upload
  unsigned int work;            // tile counter of the persistent pair kernels
  int launches;
  unsigned long long closure_eval, closure_fallback;  // closure evaluations / Smagorinsky fallbacks
  int nl_rest;    // particles the neighbour-list scan handles one per lane (set by the sort)
  // neighbour lists with a skin (FP32C form, Options::skin > 0): the cell sort
  // and the lists are rebuilt only when a particle has moved half the skin
  int rebuild;             // this step sorts and lists (always, without a skin)
  int force_rebuild;       // the next step must (upload, a particle left, a patch, an export's sort)
  unsigned int disp2_bits; // largest squared displacement since the last rebuild (FP32 bits)
  unsigned int rebuilds;   // steps that sorted and listed since upload
};

// A double's value in FP32 (truncated, not rounded) from its bits on the
// integer pipe: the estimates below need ~1e-6 relative accuracy, and a
// double-to-float conversion instruction runs on the FP64 pipe. Finite
// inputs; magnitudes outside FP32's normal range give 0 or infinity.
PSPH_D float d2f_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  const unsigned sign = hi & 0x80000000u;
  if (e <= 0) return __int_as_float((int)sign);
  if (e >= 255) return __int_as_float((int)(sign | 0x7f800000u));
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
  return __int_as_float((int)(sign | ((unsigned)e << 23) | m));
}

// Double to float, rounded to nearest even (IEEE 754), on the integer pipe:
// the same value as (float)x, without the FP64-pipe conversion instruction.
// The 52-bit significand keeps its top 23 bits; the 29 dropped bits round up
// past half, or at exactly half when the kept part is odd (a carry into the
// exponent is the next binade). Magnitudes outside [2^-74, 2^127) (the top
// binade may round to infinity, whose residual is infinite), infinities and
// NaN take the conversion instruction.
// d2f_split also returns lo = (float)(x - (double)hi), the rounding residual
// x - hi (exact in FP64: the dropped bits, or minus their complement to the
// next unit when hi rounded up) as float(+-bits) * 2^(E-1075), one rounding
// of an integer below 2^29 and an exact power-of-two scaling in FP32's normal
// range.
__host__ __device__ inline unsigned long long psph_dbits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
__host__ __device__ inline float psph_fbits(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, sizeof f);
  return f;
#endif
}

__host__ __device__ inline float d2f_split(double x, float* lo) {
  const unsigned long long b = psph_dbits(x);
  const unsigned E = (unsigned)(b >> 52) & 0x7ffu;
  if (E < 949u || E > 1149u) {
    const float h = (float)x;
    if (lo) *lo = (float)(x - (double)h);
    return h;
  }
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long m = b & 0xfffffffffffffull;
  const unsigned keep = (unsigned)(m >> 29), rem = (unsigned)m & 0x1fffffffu;
  const bool up = rem > 0x10000000u || (rem == 0x10000000u && (keep & 1u));
  const unsigned hb = sign | (((E - 896u) << 23) + keep + (up ? 1u : 0u));
  if (lo) {
    const float scale = psph_fbits((E - 948u) << 23);  // 2^(E-1075)
    int q = (int)(up ? rem - 0x20000000u : rem);
    if (sign) q = -q;
    *lo = (float)q * scale;  // +0 when exact, as x - (double)hi gives
  }
  return psph_fbits(hb);
}
__host__ __device__ inline float d2f_rn(double x) { return d2f_split(x, nullptr); }

struct GridDev {
  double blpf[3], trpr[3], cell_size[3], dom_size[3];
  double hmax, cellfac;
  int nc[3];      // real cells per axis (a periodic axis drops the reference's 2 ghost columns)
  int cn_ref[3];  // Domain::CellNo (ghost columns included)
  int periodic[3];
  int ncells;     // nc[0]*nc[1]*nc[2]
  int cell_base;  // first global cell id of this instance
  float inv_cell_size32[3];  // 1 / cell_size in FP32 (cell-index estimate of the sort)
  float cell_size32[3];      // cell_size rounded to FP32 (on the host)
  float cellfac2_32;         // Cellfac^2 in FP32
  float skin_disp2;          // with a skin: (half the skin)^2, the displacement that forces a rebuild
};

// ---------------------------------------------------------------------------
// SPH kernels (Source/Functions.cpp:25-186), evaluated without pow():
// rewritten with products and the reciprocal of r; differences from the
// reference are rounding-level (checked by the parity tests at 1e-12).
// ---------------------------------------------------------------------------
template <int DIM, int KT>
struct Kern {
  // normalisation: W = cw/h^DIM f(q); GradKernel, LaplaceKernel and
  // SecDerivativeKernel carry cw/h^(DIM+2).
  static constexpr double cw() {
    return KT == 0 ? (DIM == 2 ? 10.0 / (7.0 * kPi) : 1.0 / kPi)
         : KT == 1 ? (DIM == 2 ? 7.0 / (4.0 * kPi) : 7.0 / (8.0 * kPi))
                   : (DIM == 2 ? 7.0 / (478.0 * kPi) : 1.0 / (120.0 * kPi));
  }
  static constexpr double support() { return KT == 2 ? 3.0 : 2.0; }

  // Kernel W(q,h) with cwh = cw/h^DIM.
  static PSPH_HD double W(double q, double cwh) {
    if (KT == 0) {
      if (q < 1.0) return cwh * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
      if (q < 2.0) { double t = 2.0 - q; return cwh * (0.25 * t * t * t); }
      return 0.0;
    } else if (KT == 1) {
      if (q < 2.0) { double t = 1.0 - 0.5 * q; double t2 = t * t; return cwh * (t2 * t2) * (2.0 * q + 1.0); }
      return 0.0;
    } else {
      double a = 3.0 - q, b = 2.0 - q, c = 1.0 - q;
      double a2 = a * a, b2 = b * b, c2 = c * c;
      if (q < 1.0) return cwh * (a2 * a2 * a - 6.0 * b2 * b2 * b + 15.0 * c2 * c2 * c);
      if (q < 2.0) return cwh * (a2 * a2 * a - 6.0 * b2 * b2 * b);
      if (q < 3.0) return cwh * (a2 * a2 * a);
      return 0.0;
    }
  }
  // GradKernel (1/r dW/dr) with cwg = cw/h^(DIM+2), inv_q = 1/q (unused at q==0).
  static PSPH_HD double GK(double q, double inv_q, double cwh1) {
    if (KT == 0) {
      if (q < 1.0) return cwh1 * (-3.0 + 2.25 * q);
      if (q < 2.0) { double t = 2.0 - q; return cwh1 * inv_q * (-0.75 * t * t); }
      return 0.0;
    } else if (KT == 1) {
      if (q < 2.0) { double t = 1.0 - 0.5 * q; return cwh1 * -5.0 * (t * t * t); }
      return 0.0;
    } else {
      double a = 3.0 - q, b = 2.0 - q, c = 1.0 - q;
      double a2 = a * a, b2 = b * b, c2 = c * c;
      if (q == 0.0) return cwh1 * (20.0 * a2 * a - 120.0 * b2 * b + 300.0 * c2 * c);
      if (q < 1.0) return cwh1 * inv_q * (-5.0 * a2 * a2 + 30.0 * b2 * b2 - 75.0 * c2 * c2);
      if (q < 2.0) return cwh1 * inv_q * (-5.0 * a2 * a2 + 30.0 * b2 * b2);
      if (q < 3.0) return cwh1 * inv_q * (-5.0 * a2 * a2);
      return 0.0;
    }
  }
  // SecDerivativeKernel with cwh2 = cw/h^(DIM+2) (same constant as GK).
  static PSPH_HD double D2(double q, double cwh2) {
    if (KT == 0) {
      if (q < 1.0) return cwh2 * (-3.0 + 4.5 * q);
      if (q < 2.0) return cwh2 * (1.5 * (2.0 - q));
      return 0.0;
    } else if (KT == 1) {
      if (q < 2.0) { double t = 1.0 - 0.5 * q; return cwh2 * (t * t) * (10.0 * q - 5.0); }
      return 0.0;
    } else {
      double a = 3.0 - q, b = 2.0 - q, c = 1.0 - q;
      if (q < 1.0) return cwh2 * (20.0 * a * a * a - 120.0 * b * b * b + 300.0 * c * c * c);
      if (q < 2.0) return cwh2 * (20.0 * a * a * a - 120.0 * b * b * b);
      if (q < 3.0) return cwh2 * (20.0 * a * a * a);
      return 0.0;
    }
  }
  // LaplaceKernel = D2 + (DIM-1)/q * (first derivative / h^2 form), with cwh2.
  static PSPH_HD double Lap(double q, double inv_q, double cwh2) {
    double first;  // dW/dq / q (per C/h^(DIM+2))
    if (KT == 0) {
      if (q < 1.0) first = (-3.0 + 2.25 * q);
      else if (q < 2.0) { double t = 2.0 - q; first = inv_q * (-0.75 * t * t); }
      else return 0.0;
    } else if (KT == 1) {
      if (q < 2.0) { double t = 1.0 - 0.5 * q; first = -5.0 * t * t * t; }
      else return 0.0;
    } else {
      double a = 3.0 - q, b = 2.0 - q, c = 1.0 - q;
      double a2 = a * a, b2 = b * b, c2 = c * c;
      if (q < 1.0) first = inv_q * (-5.0 * a2 * a2 + 30.0 * b2 * b2 - 75.0 * c2 * c2);
      else if (q < 2.0) first = inv_q * (-5.0 * a2 * a2 + 30.0 * b2 * b2);
      else if (q < 3.0) first = inv_q * (-5.0 * a2 * a2);
      else return 0.0;
    }
    return D2(q, cwh2) + cwh2 * (DIM - 1.0) * first;
  }
};

// Kernel value with runtime kernel type (used off the hot loop).
template <int DIM>
PSPH_HD double kernel_w_rt(int kt, double q, double h) {
  double hd = (DIM == 2) ? h * h : h * h * h;
  switch (kt) {
    case 0: return Kern<DIM, 0>::W(q, Kern<DIM, 0>::cw() / hd);
    case 1: return Kern<DIM, 1>::W(q, Kern<DIM, 1>::cw() / hd);
    default: return Kern<DIM, 2>::W(q, Kern<DIM, 2>::cw() / hd);
  }
}

// EOS / SoundSpeed / DensitySolid (Source/Functions.cpp:188-264).
PSPH_HD double pow7(double x) { double x2 = x * x; double x3 = x2 * x; return x3 * x3 * x; }
PSPH_HD double pow6(double x) { double x2 = x * x; return x2 * x2 * x2; }

PSPH_HD double eos(int eq, double cs, double p0, double rho, double rho0) {
  switch (eq) {
    case 0: return p0 + (cs * cs) * (rho - rho0);
    case 1: return p0 + (rho0 * cs * cs / 7.0) * (pow7(rho / rho0) - 1.0);
    default: return (cs * cs) * rho;
  }
}
PSPH_HD double sound_speed(int eq, double cs, double rho, double rho0) {
  if (eq == 1) return sqrt((cs * cs) * pow6(rho / rho0));
  return cs;
}
PSPH_HD double density_solid(int eq, double cs, double p0, double p, double rho0) {
  switch (eq) {
    case 0: return (p - p0) / (cs * cs) + rho0;
    case 1: return pow(((p - p0) * (7.0 / (rho0 * cs * cs)) + 1.0), 1.0 / 7.0) * rho0;
    default: return p / (cs * cs);
  }
}

// ---------------------------------------------------------------------------
// Cell indexing
// ---------------------------------------------------------------------------
PSPH_HD int cell_linear(const GridDev& g, int cx, int cy, int cz) { return (cz * g.nc[1] + cy) * g.nc[0] + cx; }

}  // namespace psph
