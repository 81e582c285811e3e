/*
 * SPH::Particle with the reference's public field names and constructor
 * defaults (Source/Particle.h:29-149, Source/Particle.cpp:25-117), as the host
 * object a driver fills before Domain::Solve. The state lives on the GPU while
 * Solve runs; Domain copies it back into these objects at output times and at
 * the end.
 */
#ifndef PERSIANSPH_PARTICLE_H
#define PERSIANSPH_PARTICLE_H

#include "matvec.h"

namespace SPH {

class Particle {
 public:
  Particle(int Tag, Vec3_t const& x0, Vec3_t const& v0, double Mass0, double Density0, double h0, bool Fixed)
      : IsFree(!Fixed), ID(Tag), x(x0), v(v0), Density(Density0), RefDensity(Density0), Mass(Mass0), h(h0),
        V(Mass0 / Density0) {}

  // flags and identifiers
  bool IsFree;
  bool NoSlip = false;
  bool Shepard = false;
  bool LES = false;
  int ID;
  int Material = 0;
  int PresEq = 0;
  size_t VisM = 0;
  size_t Fail = 0;
  size_t ShepardStep = 40;
  size_t ShepardCounter = 0;
  bool FirstStep = true;
  int ct = 0;

  // kinematics
  Vec3_t x, v;
  Vec3_t va, vb, a, NSv, VXSPH;

  // density, pressure, mass
  double Density;
  double Densitya = 0.0, Densityb = 0.0, dDensity = 0.0;
  double RefDensity;
  double Pressure = 0.0;
  double Mass;
  double h;
  double FPMassC = 1.0;

  // fluid
  double Cs = 0.0, P0 = 0.0;
  double Alpha = 0.0, Beta = 0.0;
  double Mu = 0.0, MuRef = 0.0, T0 = 0.0, m = 300.0, CSmag = 0.17;
  double ShearRate = 0.0, SBar = 0.0;
  double TI = 0.0, TIn = 4.0, TIInitDist = 0.0;
  double ZWab = 0.0, SumDen = 0.0, SumKernel = 0.0;

  // solid / soil
  double G = 0.0, K = 0.0, c = 0.0, phi = 0.0, psi = 0.0, Sigmay = 0.0;
  Mat3_t Sigma, Sigmaa, Sigmab, ShearStress, ShearStressa, ShearStressb, Strain, Straina, Strainb;
  Mat3_t StrainRate, RotationRate, TIR;

  // soil-water interaction (fluid and soil in one domain)
  size_t SeepageType = 0;
  bool VarPorosity = false, IsSat = false;
  double n0 = 0.0, k = 0.0, k2 = 0.0, d = 0.0, RhoF = 0.0;
  double V;         // volume: Mass / RefDensity at construction
  double S = 0.0;   // SWIType 1: surface-erosion velocity derivative of the last step
  size_t InOut = 0; // in/out-flow boundary: 1 in the in-flow zone, 2 in the out-flow zone
};

}  // namespace SPH

#endif  // PERSIANSPH_PARTICLE_H
