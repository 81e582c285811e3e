/*
 * SPH::Domain for GB300: the reference's driver-facing API (Source/Domain.h)
 * with the per-step body of Solve on the GPU through the C ABI (psph.h).
 *
 * A driver written for the reference (`#include "Domain.h"`, fill
 * dom.Particles, call dom.Solve) compiles unchanged with
 *   g++ -std=c++14 driver.cpp -I include/persiansph -I include
 *       -L persiansph_gb300/_build -lpsph_gb300
 * Kept: the enums and selectors (Kernel_Set, Viscosity_Eq_Set,
 * Gradient_Approach_Set), AddSingleParticle / AddBoxLength / AddBoxNo /
 * DelParticles, the public data drivers set (Particles, Dimension, Gravity,
 * Scheme, BC.Periodic, XSPH, InitialDist, DomMax/DomMin, sqrt_h_a, Nproc,
 * SWIType, FSI, the in/out-flow settings of BC) and the hooks (GeneralBefore,
 * GeneralAfter, UserOutput, InCon / OutCon / AllCon). A user InCon / OutCon
 * runs on the host once per in/out-flow particle per step, as in the
 * reference; particles an in/out-flow boundary appends become new Particle
 * objects at the end of Particles when they are copied back.
 * Solve (Source/Domain.cpp:1735-1797) keeps its outer loop over output times;
 * each stretch between outputs is one psph_step call, and the particles are
 * copied back into dom.Particles at every output time and at the end.
 *
 * Differences a driver can see:
 *  - GeneralBefore / GeneralAfter run on the host every step, where the
 *    reference calls them (after the neighbour search; after the forces):
 *    the particles are copied back into dom.Particles (with Time), the hook
 *    runs, and what it changed goes back to the device (psph_patch). That
 *    costs two copies of the particles per step; a constant acceleration is
 *    cheaper as Domain::BodyForce, which the pair kernels add on the device.
 *    A hook may change particle parameters (cohesion, friction angle, ...)
 *    but not switch on a pair term no particle had (psph_patch says which).
 *  - Output: with a file key, Solve writes the reference's snapshots
 *    (WriteXDMF: <key>_Initial, then <key>_0001, ... at each output time) as
 *    <name>.bin + <name>.xmf, the same datasets as the reference's <name>.hdf5
 *    in a raw little-endian file the .xmf points at (HDF5 is not linked).
 *    With the default UserOutput the snapshot is taken on the device at the
 *    reference's output point (after the step's forces, before its update)
 *    and written while the next steps run; a driver-set UserOutput runs on the
 *    host on the particles copied back at the output time (accelerations of
 *    the step before). OutputHook (an addition) is called at output times with
 *    the particles copied back.
 *  - Additions: Precision (PSPH_FP64 / PSPH_FP32C), BodyForce,
 *    WallPressureMode, ShepardStep, Time (public), OutputHook.
 *  - Nproc is accepted and ignored (the work runs on the GPU).
 *
 * AddBoxLength's lattice arithmetic runs in the driver's own compilation. Arm
 * compilers fuse x0 + i*2r into one FMA by default, which moves positions by
 * an ulp against an x86 build of the reference; add -ffp-contract=off for
 * bit-identical lattices on both.
 */
#ifndef PERSIANSPH_DOMAIN_H
#define PERSIANSPH_DOMAIN_H

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <iostream>
#include <utility>
#include <vector>

#include "Particle.h"
#include "psph.h"

enum Kernels_Type { Qubic_Spline = 0, Quintic = 1, Quintic_Spline = 2 };
enum Viscosity_Eq_Type { Morris = 0, Shao = 1, Incompressible_Full = 2, Takeda = 3 };
enum Gradient_Type { Squared_density = 0, Multiplied_density = 1 };

namespace SPH {

// Boundary (Source/Boundary_Condition.h:25-55): Periodic, and the in/out-flow
// settings (InOutFlow, inv/inDensity, outv/outDensity, allv/allDensity,
// cellfac, MassConservation) Solve hands to the device.
class Boundary {
 public:
  double inDensity = 0.0, outDensity = 0.0, allDensity = 0.0;
  Vec3_t inv, outv, allv;
  bool Periodic[3] = {false, false, false};
  int InOutFlow = 0;
  double InFlowLoc1 = 0.0, InFlowLoc2 = 0.0, InFlowLoc3 = 0.0, OutFlowLoc = 0.0;
  double cellfac = 3.9;
  int inoutcounter = 0;
  bool MassConservation = false;
};

class Domain;
inline void General(Domain&) {}
inline void OutPut(Particle*, double& a, double& b, double& c) { a = b = c = 0.0; }
// the default in/out-flow hooks (Source/Domain.cpp:35-51)
inline void InFlowCon(Vec3_t&, Vec3_t& Vel, double& Den, Boundary& bdry) {
  Vel = bdry.inv;
  Den = bdry.inDensity;
}
inline void OutFlowCon(Vec3_t&, Vec3_t& Vel, double& Den, Boundary& bdry) {
  Vel = bdry.outv;
  Den = bdry.outDensity;
}
inline void AllFlowCon(Vec3_t&, Vec3_t& Vel, double& Den, Boundary& bdry) {
  Vel = bdry.allv;
  Den = bdry.allDensity;
}

class Domain {
 public:
  typedef void (*PtVel)(Vec3_t& position, Vec3_t& Vel, double& Den, Boundary& bdry);
  typedef void (*PtOut)(Particle* Particles, double& Prop1, double& Prop2, double& Prop3);
  typedef void (*PtDom)(Domain& dom);

  Domain() {
    OutputName[0] = "Property1";
    OutputName[1] = "Property2";
    OutputName[2] = "Property3";
    DomMax = -100000000000.0;
    DomMin = 100000000000.0;
  }
  ~Domain() {
    for (Particle* p : Particles) delete p;
  }
  Domain(const Domain&) = delete;
  Domain& operator=(const Domain&) = delete;

  // -- selectors (Source/Domain.cpp:117-131) ----------------------------------
  void Kernel_Set(Kernels_Type const& KT) { KernelType = (int)KT; }
  void Viscosity_Eq_Set(Viscosity_Eq_Type const& VQ) { VisEq = (int)VQ; }
  void Gradient_Approach_Set(Gradient_Type const& GT) { GradientType = (int)GT; }

  // -- particle generation ----------------------------------------------------
  void AddSingleParticle(int tag, Vec3_t const& x, double Mass, double Density, double h, bool Fixed) {
    Particles.Push(new Particle(tag, x, Vec3_t(0, 0, 0), Mass, Density, h, Fixed));
  }
  void AddBoxLength(int tag, Vec3_t const& V, double Lx, double Ly, double Lz, double r, double Density, double h,
                    int type, int rotation, bool random, bool Fixed);
  void AddBoxNo(int tag, Vec3_t const& V, size_t nx, size_t ny, size_t nz, double r, double Density, double h,
                int type, int rotation, bool random, bool Fixed);
  void DelParticles(int const& Tags);

  // -- solve ------------------------------------------------------------------
  void Solve(double tf, double dt, double dtOut, char const* TheFileKey, size_t maxidx);

  // -- data (Source/Domain.h:93-145) --------------------------------------------
  Array<Particle*> Particles;
  double R = 0.0;
  double sqrt_h_a = 0.0025;
  int Dimension = 2;
  Vec3_t Gravity;
  size_t SWIType = 0;
  bool FSI = false;
  double XSPH = 0.0;
  double InitialDist = 0.0;
  size_t Nproc = 1;
  Boundary BC;
  PtOut UserOutput = &OutPut;
  PtVel InCon = &InFlowCon;
  PtVel OutCon = &OutFlowCon;
  PtVel AllCon = &AllFlowCon;
  Vec3_t DomMax, DomMin;
  PtDom GeneralBefore = &General;
  PtDom GeneralAfter = &General;
  size_t Scheme = 0;
  String OutputName[3];
  double Time = 0.0;

  // -- additions of this build ------------------------------------------------
  int Precision = PSPH_FP64;            // PSPH_FP32C: FP32 pair arithmetic, compensated sums
  Vec3_t BodyForce;                     // constant acceleration of free particles, on the device
  int WallPressureMode = PSPH_WALLP_REFERENCE;
  int ShepardStep = 40;                 // Particle::ShepardStep, uniform over particles
  std::function<void(Domain&, size_t)> OutputHook;  // called at output times (particles copied back)

 private:
  int KernelType = 0, VisEq = 0, GradientType = 0;

  // host SoA image of the particles for the C ABI
  struct Pack {
    std::vector<int32_t> id, material, is_free, no_slip, pres_eq, shepard, les, vis_m, fail;
    std::vector<int32_t> seepage_type, var_porosity, is_sat, in_out;
    std::vector<double> vec[7];     // x v va vb a nsv vxsph
    std::vector<double> sca[38];
    std::vector<double> ten[12];
    std::vector<double> s;          // Particle::S
    psph_particles view;
  };
  void pack(Pack& pk) const;
  void unpack(const Pack& pk);
  // GeneralBefore / GeneralAfter inside a step (psph_set_step_hooks): Solve
  // sets hook_run_ to copy the particles back, call the hook and patch them
  std::function<void(int)> hook_run_;
  std::exception_ptr hook_error_;
  static int step_hook(psph_ctx*, int where, void* u) {
    Domain* d = static_cast<Domain*>(u);
    try {
      d->hook_run_(where);
      return 0;
    } catch (...) {
      d->hook_error_ = std::current_exception();
      return 1;
    }
  }
  void WholeVelocity();
  // a user InCon / OutCon called by the library (psph_flow_fn) for one particle
  static void flow_hook(PtVel hook, Domain* d, const double* x, double* v, double* den) {
    Vec3_t X(x[0], x[1], x[2]), V(0, 0, 0);
    double D = 0.0;
    hook(X, V, D, d->BC);
    for (int k = 0; k < 3; ++k) v[k] = V(k);
    *den = D;
  }
  static void in_flow_hook(const double* x, double* v, double* den, void* u) {
    Domain* d = static_cast<Domain*>(u);
    flow_hook(d->InCon, d, x, v, den);
  }
  static void out_flow_hook(const double* x, double* v, double* den, void* u) {
    Domain* d = static_cast<Domain*>(u);
    flow_hook(d->OutCon, d, x, v, den);
  }
  static void check(psph_status st, psph_ctx* ctx) {
    if (st != PSPH_OK) {
      const std::string msg = psph_last_error(ctx);
      throw new Fatal("%s", msg.c_str());
    }
  }
};

// ---- field tables: SPH::Particle member <-> psph_particles array ----------------
namespace detail {
struct VecF { Vec3_t Particle::*m; double* psph_particles::*p; };
struct ScaF { double Particle::*m; double* psph_particles::*p; };
struct TenF { Mat3_t Particle::*m; double* psph_particles::*p; };
inline const VecF* vec_fields() {
  static const VecF f[7] = {{&Particle::x, &psph_particles::x},     {&Particle::v, &psph_particles::v},
                            {&Particle::va, &psph_particles::va},   {&Particle::vb, &psph_particles::vb},
                            {&Particle::a, &psph_particles::a},     {&Particle::NSv, &psph_particles::nsv},
                            {&Particle::VXSPH, &psph_particles::vxsph}};
  return f;
}
inline const ScaF* sca_fields() {
  static const ScaF f[38] = {
      {&Particle::Density, &psph_particles::density},       {&Particle::Densitya, &psph_particles::densitya},
      {&Particle::Densityb, &psph_particles::densityb},     {&Particle::dDensity, &psph_particles::ddensity},
      {&Particle::Pressure, &psph_particles::pressure},     {&Particle::Mass, &psph_particles::mass},
      {&Particle::h, &psph_particles::h},                   {&Particle::Cs, &psph_particles::cs},
      {&Particle::P0, &psph_particles::p0},                 {&Particle::RefDensity, &psph_particles::ref_density},
      {&Particle::FPMassC, &psph_particles::fpmassc},       {&Particle::Alpha, &psph_particles::alpha},
      {&Particle::Beta, &psph_particles::beta},             {&Particle::Mu, &psph_particles::mu},
      {&Particle::MuRef, &psph_particles::mu_ref},          {&Particle::T0, &psph_particles::t0},
      {&Particle::m, &psph_particles::bingham_m},           {&Particle::CSmag, &psph_particles::csmag},
      {&Particle::TI, &psph_particles::ti},                 {&Particle::TIn, &psph_particles::tin},
      {&Particle::TIInitDist, &psph_particles::ti_init_dist}, {&Particle::G, &psph_particles::g_mod},
      {&Particle::K, &psph_particles::k_mod},               {&Particle::Sigmay, &psph_particles::sigmay},
      {&Particle::c, &psph_particles::cohesion},            {&Particle::phi, &psph_particles::phi},
      {&Particle::psi, &psph_particles::psi},               {&Particle::ZWab, &psph_particles::zwab},
      {&Particle::SumDen, &psph_particles::sumden},         {&Particle::SumKernel, &psph_particles::sumkernel},
      {&Particle::ShearRate, &psph_particles::shear_rate},  {&Particle::SBar, &psph_particles::sbar},
      // soil-water interaction; k and k2 last: an upload reads them, a download leaves them
      {&Particle::n0, &psph_particles::n0},                 {&Particle::d, &psph_particles::d},
      {&Particle::RhoF, &psph_particles::rho_f},            {&Particle::V, &psph_particles::volume},
      {&Particle::k, &psph_particles::k},                   {&Particle::k2, &psph_particles::k2}};
  return f;
}
inline const TenF* ten_fields() {
  static const TenF f[12] = {
      {&Particle::Sigma, &psph_particles::sigma},               {&Particle::Sigmaa, &psph_particles::sigmaa},
      {&Particle::Sigmab, &psph_particles::sigmab},             {&Particle::ShearStress, &psph_particles::shear_stress},
      {&Particle::ShearStressa, &psph_particles::shear_stressa}, {&Particle::ShearStressb, &psph_particles::shear_stressb},
      {&Particle::Strain, &psph_particles::strain},             {&Particle::Straina, &psph_particles::straina},
      {&Particle::Strainb, &psph_particles::strainb},           {&Particle::StrainRate, &psph_particles::strain_rate},
      {&Particle::RotationRate, &psph_particles::rotation_rate}, {&Particle::TIR, &psph_particles::tir}};
  return f;
}
// while (p <= limit) loop count with p = start, then p = pos(i) (the generators' loop form)
template <class F>
inline size_t lattice_count(double start, double limit, F pos) {
  size_t i = 0;
  double p = start;
  while (p <= limit) {
    ++i;
    p = pos(i);
  }
  return i;
}
}  // namespace detail

inline void Domain::pack(Pack& pk) const {
  const size_t n = Particles.Size();
  std::memset(&pk.view, 0, sizeof pk.view);
  pk.view.n = (int64_t)n;
  auto ints = [&](std::vector<int32_t>& v, int32_t* psph_particles::*p, auto get) {
    v.resize(n);
    for (size_t i = 0; i < n; ++i) v[i] = (int32_t)get(*Particles[i]);
    pk.view.*p = v.data();
  };
  ints(pk.id, &psph_particles::id, [](const Particle& q) { return q.ID; });
  ints(pk.material, &psph_particles::material, [](const Particle& q) { return q.Material; });
  ints(pk.is_free, &psph_particles::is_free, [](const Particle& q) { return q.IsFree ? 1 : 0; });
  ints(pk.no_slip, &psph_particles::no_slip, [](const Particle& q) { return q.NoSlip ? 1 : 0; });
  ints(pk.pres_eq, &psph_particles::pres_eq, [](const Particle& q) { return q.PresEq; });
  ints(pk.shepard, &psph_particles::shepard, [](const Particle& q) { return q.Shepard ? 1 : 0; });
  ints(pk.les, &psph_particles::les, [](const Particle& q) { return q.LES ? 1 : 0; });
  ints(pk.vis_m, &psph_particles::vis_m, [](const Particle& q) { return (int)q.VisM; });
  ints(pk.fail, &psph_particles::fail, [](const Particle& q) { return (int)q.Fail; });
  ints(pk.seepage_type, &psph_particles::seepage_type, [](const Particle& q) { return (int)q.SeepageType; });
  ints(pk.var_porosity, &psph_particles::var_porosity, [](const Particle& q) { return q.VarPorosity ? 1 : 0; });
  ints(pk.is_sat, &psph_particles::is_sat, [](const Particle& q) { return q.IsSat ? 1 : 0; });
  ints(pk.in_out, &psph_particles::in_out, [](const Particle& q) { return (int)q.InOut; });
  for (int f = 0; f < 7; ++f) {
    const detail::VecF& F = detail::vec_fields()[f];
    pk.vec[f].resize(3 * n);
    for (size_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) pk.vec[f][3 * i + d] = ((*Particles[i]).*F.m)(d);
    pk.view.*F.p = pk.vec[f].data();
  }
  for (int f = 0; f < 38; ++f) {
    const detail::ScaF& F = detail::sca_fields()[f];
    pk.sca[f].resize(n);
    for (size_t i = 0; i < n; ++i) pk.sca[f][i] = (*Particles[i]).*F.m;
    pk.view.*F.p = pk.sca[f].data();
  }
  pk.s.resize(n);
  for (size_t i = 0; i < n; ++i) pk.s[i] = Particles[i]->S;
  pk.view.s = pk.s.data();
  for (int f = 0; f < 12; ++f) {
    const detail::TenF& F = detail::ten_fields()[f];
    pk.ten[f].resize(9 * n);
    for (size_t i = 0; i < n; ++i) std::memcpy(&pk.ten[f][9 * i], ((*Particles[i]).*F.m).data(), 9 * sizeof(double));
    pk.view.*F.p = pk.ten[f].data();
  }
}

// Copies a downloaded image (original order, leavers removed) back into the
// particle objects; particles that left the domain are deleted as
// CheckParticleLeave does (Source/Domain.cpp:517-547). The per-particle
// constants come back too: an in/out-flow boundary recycles a particle with
// the in-flow's ID, material and parameters (Source/Domain.cpp:1363-1395).
inline void Domain::unpack(const Pack& pk) {
  const size_t n = (size_t)pk.view.n;
  for (size_t i = 0; i < n; ++i) {
    Particle& q = *Particles[i];
    q.ID = pk.id[i];
    q.Material = pk.material[i];
    q.IsFree = pk.is_free[i] != 0;
    q.NoSlip = pk.no_slip[i] != 0;
    q.PresEq = pk.pres_eq[i];
    q.Shepard = pk.shepard[i] != 0;
    q.LES = pk.les[i] != 0;
    q.VisM = (size_t)pk.vis_m[i];
    q.Fail = (size_t)pk.fail[i];
    q.SeepageType = (size_t)pk.seepage_type[i];
    q.VarPorosity = pk.var_porosity[i] != 0;
    q.InOut = (size_t)pk.in_out[i];
    for (int f = 0; f < 7; ++f) {
      const detail::VecF& F = detail::vec_fields()[f];
      for (int d = 0; d < 3; ++d) (q.*F.m)(d) = pk.vec[f][3 * i + d];
    }
    for (int f = 0; f < 36; ++f) q.*(detail::sca_fields()[f].m) = pk.sca[f][i];  // not k, k2
    q.IsSat = pk.is_sat[i] != 0;
    q.S = pk.s[i];
    for (int f = 0; f < 12; ++f) std::memcpy((q.*(detail::ten_fields()[f].m)).data(), &pk.ten[f][9 * i], 9 * sizeof(double));
  }
}

inline void Domain::AddBoxLength(int tag, Vec3_t const& V, double Lx, double Ly, double Lz, double r, double Density,
                                 double h, int type, int rotation, bool random, bool Fixed) {
  // Source/Domain.cpp:294-495: hexagonal (type 0) or cubic (type 1) lattice
  if (!(type == 0 || type == 1)) throw new Fatal("Packing Type is out of range. Please correct it and run again");
  if (!(rotation == 0 || rotation == 90))
    throw new Fatal("Packing Rotation Angle is out of range. Please correct it and run again");
  const size_t pre = Particles.Size();
  const double sq3 = std::sqrt(3.0);
  std::vector<Vec3_t> pts;
  double mass = 0.0;
  if (Dimension == 3) {
    if (type == 0) {
      const double dz = 2.0 * std::sqrt(6.0) / 3.0;
      for (int k = 0;; ++k) {
        const double zp = (k == 0) ? V(2) : V(2) + (dz * k + 1) * r;
        if (!(zp <= V(2) + Lz - r)) break;
        for (int j = 0;; ++j) {
          const double yp = (j == 0) ? V(1) : V(1) + (sq3 * (j + (1.0 / 3.0) * (k % 2)) + 1) * r;
          if (!(yp <= V(1) + Ly - r)) break;
          const bool odd = (k % 2 != 0) && (j % 2 != 0);
          const int off = (j % 2) + (k % 2) + (odd ? -1 : 1);
          const size_t ni = detail::lattice_count(V(0), V(0) + Lx - r, [&](size_t i) { return V(0) + (2.0 * i + off) * r; });
          for (size_t i = 0; i < ni; ++i)
            pts.push_back(Vec3_t(V(0) + (2 * (double)i + off) * r, V(1) + (sq3 * (j + (1.0 / 3.0) * (k % 2)) + 1) * r,
                                 V(2) + (dz * k + 1) * r));
        }
      }
    } else {
      const size_t nx = detail::lattice_count(V(0), V(0) + Lx - r, [&](size_t i) { return V(0) + (2.0 * i + 1) * r; });
      const size_t ny = detail::lattice_count(V(1), V(1) + Ly - r, [&](size_t j) { return V(1) + (2.0 * j + 1) * r; });
      const size_t nz = detail::lattice_count(V(2), V(2) + Lz - r, [&](size_t k) { return V(2) + (2.0 * k + 1) * r; });
      for (size_t k = 0; k < nz; ++k)
        for (size_t j = 0; j < ny; ++j)
          for (size_t i = 0; i < nx; ++i)
            pts.push_back(Vec3_t(V(0) + (2.0 * i + 1) * r, V(1) + (2.0 * j + 1) * r, V(2) + (2.0 * k + 1) * r));
    }
  } else {
    if (type == 0) {
      mass = (sq3 * r * r) * Density;
      if (rotation == 0) {
        for (int j = 0;; ++j) {
          const double yp = (j == 0) ? V(1) : V(1) + (sq3 * j + 1) * r;
          if (!(yp <= V(1) + Ly - r)) break;
          const int off = (j % 2) + 1;
          const size_t ni = detail::lattice_count(V(0), V(0) + Lx - r, [&](size_t i) { return V(0) + (2.0 * i + off) * r; });
          for (size_t i = 0; i < ni; ++i) pts.push_back(Vec3_t(V(0) + (2 * (double)i + off) * r, V(1) + (sq3 * j + 1) * r, 0.0));
        }
      } else {
        for (int i = 0;; ++i) {
          const double xp = (i == 0) ? V(0) : V(0) + (sq3 * i + 1) * r;
          if (!(xp <= V(0) + Lx - r)) break;
          const int off = (i % 2) + 1;
          const size_t nj = detail::lattice_count(V(1), V(1) + Ly - r, [&](size_t j) { return V(1) + (2.0 * j + off) * r; });
          for (size_t j = 0; j < nj; ++j) pts.push_back(Vec3_t(V(0) + (sq3 * i + 1) * r, V(1) + (2 * (double)j + off) * r, 0.0));
        }
      }
    } else {
      mass = random ? (sq3 * r * r) * Density : 2.0 * r * 2.0 * r * Density;
      const size_t nx = detail::lattice_count(V(0), V(0) + Lx - r, [&](size_t i) { return V(0) + (2.0 * i + 1) * r; });
      const size_t ny = detail::lattice_count(V(1), V(1) + Ly - r, [&](size_t j) { return V(1) + (2.0 * j + 1) * r; });
      for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i) pts.push_back(Vec3_t(V(0) + (2.0 * i + 1) * r, V(1) + (2.0 * j + 1) * r, 0.0));
    }
  }
  if (random) {  // srand(100), then rand() per jittered coordinate (Source/Domain.cpp:329-330)
    std::srand(100);
    const double qin = 0.03;
    const int ncomp = (Dimension == 3) ? 3 : 2;
    for (Vec3_t& p : pts)
      for (int d = 0; d < ncomp; ++d) p(d) = p(d) + qin * r * double(std::rand()) / RAND_MAX;
  }
  for (const Vec3_t& p : pts) Particles.Push(new Particle(tag, p, Vec3_t(0, 0, 0), mass, Density, h, Fixed));
  if (Dimension == 3 && Particles.Size() > pre) {  // 3D mass from the bounding box (Source/Domain.cpp:399-415)
    Vec3_t mx = V;
    for (size_t i = pre; i < Particles.Size(); ++i)
      for (int d = 0; d < 3; ++d)
        if (Particles[i]->x(d) > mx(d)) mx(d) = Particles[i]->x(d);
    const double m3 = ((mx(0) + r) - V(0)) * ((mx(1) + r) - V(1)) * ((mx(2) + r) - V(2)) * Density /
                      (double)(Particles.Size() - pre);
    for (size_t i = pre; i < Particles.Size(); ++i) Particles[i]->Mass = m3;
  }
  R = r;
}

inline void Domain::AddBoxNo(int tag, Vec3_t const& V, size_t nx, size_t ny, size_t nz, double r, double Density,
                             double h, int type, int rotation, bool random, bool Fixed) {
  // Source/Domain.cpp:159-292 with cubic packing; the hexagonal form takes AddBoxLength
  if (!(type == 0 || type == 1)) throw new Fatal("Packing Type is out of range. Please correct it and run again");
  if (!(rotation == 0 || rotation == 90))
    throw new Fatal("Packing Rotation Angle is out of range. Please correct it and run again");
  if (type != 1) throw new Fatal("AddBoxNo with hexagonal packing: use AddBoxLength");
  const Vec3_t L((2.0 * nx) * r + r / 10.0, (2.0 * ny) * r + r / 10.0, (2.0 * nz) * r + r / 10.0);
  AddBoxLength(tag, V, L(0), L(1), Dimension == 3 ? L(2) : 0.0, r, Density, h, type, rotation, random, Fixed);
}

inline void Domain::DelParticles(int const& Tags) {
  // Source/Domain.cpp:497-515: order-preserving removal by tag
  Array<Particle*> kept;
  for (Particle* p : Particles) {
    if (p->ID == Tags) delete p;
    else kept.Push(p);
  }
  if (kept.Size() == Particles.Size()) throw new Fatal("Domain::DelParticles: Could not find any particles to delete");
  Particles.swap(kept);
}

// WholeVelocity (Source/Domain.cpp:1636-1659): with BC.allv or BC.allDensity
// set, the free particles take what AllCon gives for their position; runs on
// the host before the upload, whose InitialChecks derives the pressure from the
// new density.
inline void Domain::WholeVelocity() {
  if (!(norm(BC.allv) > 0.0 || BC.allDensity > 0.0)) return;
  for (size_t i = 0; i < Particles.Size(); i++) {
    Vec3_t vel(0, 0, 0);
    double den = 0.0;
    AllCon(Particles[i]->x, vel, den, BC);
    if (Particles[i]->IsFree && norm(BC.allv) > 0.0) Particles[i]->v = vel;
    if (Particles[i]->IsFree && BC.allDensity > 0.0) Particles[i]->Density = den;
  }
}

inline void Domain::Solve(double tf, double dt, double dtOut, char const* TheFileKey, size_t maxidx) {
  std::cout << "\n--------------Solving---------------------------------------------------------------" << std::endl;
  const Vec3_t body = BodyForce;
  psph_config cfg;
  std::memset(&cfg, 0, sizeof cfg);
  cfg.dimension = Dimension;
  cfg.kernel_type = KernelType;
  cfg.vis_eq = VisEq;
  cfg.gradient_type = GradientType;
  cfg.scheme = (int)Scheme;
  for (int d = 0; d < 3; ++d) {
    cfg.periodic[d] = BC.Periodic[d] ? 1 : 0;
    cfg.gravity[d] = Gravity(d);
    cfg.body_force[d] = body(d);
    cfg.dom_max[d] = DomMax(d);
    cfg.dom_min[d] = DomMin(d);
  }
  cfg.shepard_step = ShepardStep;
  cfg.precision = Precision;
  cfg.wall_pressure_mode = WallPressureMode;
  cfg.xsph = XSPH;
  cfg.sqrt_h_a = sqrt_h_a;
  cfg.R = R;
  cfg.dt = dt;
  cfg.time = Time;
  cfg.swi_type = (int)SWIType;
  cfg.fsi = FSI ? 1 : 0;
  cfg.in_out_flow = BC.InOutFlow;
  cfg.mass_conservation = BC.MassConservation ? 1 : 0;
  cfg.bc_cellfac = BC.cellfac;
  cfg.initial_dist = InitialDist;
  cfg.in_density = BC.inDensity;
  cfg.out_density = BC.outDensity;
  for (int d = 0; d < 3; ++d) {
    cfg.in_v[d] = BC.inv(d);
    cfg.out_v[d] = BC.outv(d);
  }
  WholeVelocity();

  psph_ctx* ctx = nullptr;
  Pack pk;
  try {
    const psph_status cst = psph_create(&cfg, &ctx);
    check(cst, ctx);
    const bool before = GeneralBefore != &General, after = GeneralAfter != &General;
    if (before || after)  // host hooks inside every step, where the reference calls them
      check(psph_set_step_hooks(ctx, &Domain::step_hook, this,
                                (before ? PSPH_HOOK_BEFORE : 0) | (after ? PSPH_HOOK_AFTER : 0)),
            ctx);
    if (BC.InOutFlow > 0) {  // user InCon / OutCon run on the host, per in/out-flow particle
      if (InCon != &InFlowCon) check(psph_set_flow_profile(ctx, PSPH_FLOW_IN, &Domain::in_flow_hook, this), ctx);
      if (OutCon != &OutFlowCon) check(psph_set_flow_profile(ctx, PSPH_FLOW_OUT, &Domain::out_flow_hook, this), ctx);
    }
    pack(pk);
    check(psph_upload(ctx, &pk.view, 1), ctx);
    size_t idx_out = 1;
    double tout = Time;
    const bool user_props = UserOutput != &OutPut;
    const char* names[3] = {OutputName[0].CStr(), OutputName[1].CStr(), OutputName[2].CStr()};
    // UserOutput's three properties of the particles on the host, in their order
    auto write_now = [&](const String& fn) {
      std::vector<double> p1, p2, p3;
      if (user_props) {
        const size_t n = Particles.Size();
        p1.resize(n);
        p2.resize(n);
        p3.resize(n);
        for (size_t i = 0; i < n; ++i) UserOutput(Particles[i], p1[i], p2[i], p3[i]);
      }
      check(psph_output_write(ctx, fn.CStr(), names, user_props ? p1.data() : nullptr,
                              user_props ? p2.data() : nullptr, user_props ? p3.data() : nullptr),
            ctx);
    };
    if (TheFileKey != nullptr) {  // the initial state (Source/Domain.cpp:1752-1758)
      String fn;
      fn.Printf("%s_Initial", TheFileKey);
      write_now(fn);
      std::cout << "\nInitial Condition has been generated\n" << std::endl;
    }
    // the particle objects by original index (the upload's order; an in/out-flow
    // boundary appends particles with the next indices)
    std::vector<Particle*> by_orig;
    for (size_t i = 0; i < Particles.Size(); ++i) by_orig.push_back(Particles[i]);
    auto copy_back = [&]() {
      const int64_t n = psph_num_particles(ctx);
      if (n < 0) check(PSPH_ERR_CUDA, ctx);
      std::vector<int64_t> orig((size_t)std::max<int64_t>(n, 1));
      check(psph_original_index(ctx, orig.data()), ctx);
      // the survivors in order (CheckParticleLeave / InFlowBCLeave removed the
      // rest), and new objects for appended in-flow particles
      Array<Particle*> now;
      std::vector<char> alive(by_orig.size(), 0);
      bool same = (size_t)n == Particles.Size();
      for (int64_t r = 0; r < n; ++r) {
        const size_t o = (size_t)orig[(size_t)r];
        if (o >= by_orig.size()) {
          by_orig.resize(o + 1, nullptr);
          alive.resize(o + 1, 0);
        }
        if (!by_orig[o]) by_orig[o] = new Particle(0, Vec3_t(0, 0, 0), Vec3_t(0, 0, 0), 0.0, 1.0, 0.0, false);
        alive[o] = 1;
        now.Push(by_orig[o]);
        if (same && Particles[(size_t)r] != by_orig[o]) same = false;
      }
      if (!same) {
        for (size_t o = 0; o < by_orig.size(); ++o)
          if (by_orig[o] && !alive[o]) {
            delete by_orig[o];
            by_orig[o] = nullptr;
          }
        Particles.swap(now);
        pack(pk);
      }
      pk.view.n = n;
      check(psph_download(ctx, &pk.view), ctx);
      unpack(pk);
    };
    // a hook sees the particles and Time of that point of the step; its
    // changes go back with psph_patch
    hook_run_ = [&](int where) {
      copy_back();
      psph_integrator it;
      check(psph_get_integrator(ctx, &it), ctx);
      Time = it.time;
      (where == PSPH_HOOK_BEFORE ? GeneralBefore : GeneralAfter)(*this);
      pack(pk);
      check(psph_patch(ctx, &pk.view), ctx);
    };
    auto step_check = [&](psph_status st) {
      if (st != PSPH_OK && hook_error_) {
        std::exception_ptr e = hook_error_;
        hook_error_ = nullptr;
        std::rethrow_exception(e);
      }
      check(st, ctx);
    };
    while (Time < tf && idx_out <= maxidx) {
      if (Time >= tout) {
        if (OutputHook || (TheFileKey != nullptr && user_props)) copy_back();
        if (OutputHook) OutputHook(*this, idx_out);
        if (TheFileKey != nullptr) {
          String fn;
          fn.Printf("%s_%04zu", TheFileKey, idx_out);
          if (user_props) write_now(fn);
          else check(psph_output_request(ctx, fn.CStr(), names), ctx);  // taken by the next step
          std::cout << "\nOutput No. " << idx_out << " at " << Time << " has been generated" << std::endl;
        }
        idx_out++;
        tout += dtOut;
      }
      int64_t done = 0;
      step_check(psph_step(ctx, (int64_t)1 << 40, std::min(tf, tout), &done));
      psph_integrator it;
      check(psph_get_integrator(ctx, &it), ctx);
      Time = it.time;
      if (done == 0) break;
    }
    check(psph_output_flush(ctx), ctx);
    copy_back();
  } catch (...) {
    psph_destroy(ctx);
    hook_run_ = nullptr;
    throw;
  }
  psph_destroy(ctx);
  hook_run_ = nullptr;
  std::cout << "\n--------------Solving is finished---------------------------------------------------" << std::endl;
}

}  // namespace SPH

#endif  // PERSIANSPH_DOMAIN_H
