// A driver in the reference's style that writes snapshots through
// Domain::Solve's file key (the 2-Couette.cpp pattern of OutputName and
// UserOutput): the dam2d parity case of tests/golden/cases.py solved to tf
// with an output every dtOut. With a fourth argument "user" it sets a
// UserOutput of its own (velocity x, density, shear rate).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "Domain.h"

void VelocityDensityOutput(SPH::Particle* P, double& Prop1, double& Prop2, double& Prop3) {
  Prop1 = P->v(0);
  Prop2 = P->Density;
  Prop3 = P->ShearRate;
}

int main(int argc, char** argv) try {
  if (argc < 4) {
    std::printf("usage: %s file_key tf dtOut [user]\n", argv[0]);
    return 2;
  }
  const double tf = std::atof(argv[2]), dtout = std::atof(argv[3]);
  SPH::Domain dom;
  dom.Dimension = 2;
  dom.Nproc = 4;
  dom.Scheme = 0;
  dom.Viscosity_Eq_Set(Morris);
  dom.Kernel_Set(Qubic_Spline);
  dom.Gradient_Approach_Set(Squared_density);

  const double dx = 0.02, L = 0.4, H = 0.8, TL = 1.6, TH = 1.2, rho = 1000.0, g = 9.81, mu = 1.002e-3;
  const double h = 1.2 * dx, cs = 10.0 * std::sqrt(2.0 * g * H);
  dom.InitialDist = dx;
  dom.Gravity = 0.0, -g, 0.0;
  dom.AddBoxLength(1, Vec3_t(-3.0 * dx, -3.0 * dx, 0.0), 6.0 * dx + TL + dx / 10.0, 3.0 * dx + TH + dx / 10.0, 0,
                   dx / 2.0, 1.0, 1.0, 1, 0, false, false);
  for (size_t a = 0; a < dom.Particles.Size(); a++) {
    SPH::Particle* p = dom.Particles[a];
    const double xb = p->x(0), yb = p->x(1);
    const bool wall = (xb < 0.0) || (yb < 0.0) || (xb > TL);
    if (!wall && (yb > H || xb > L)) p->ID = 11;
  }
  dom.DelParticles(11);
  for (size_t a = 0; a < dom.Particles.Size(); a++) {
    SPH::Particle* p = dom.Particles[a];
    const double xb = p->x(0), yb = p->x(1);
    const bool wall = (xb < 0.0) || (yb < 0.0) || (xb > TL);
    p->h = h;
    p->Density = rho;
    p->RefDensity = rho;
    p->Cs = cs;
    p->PresEq = 1;
    p->Mu = mu;
    p->MuRef = mu;
    p->Material = 1;
    p->Alpha = 0.1;
    p->Shepard = true;
    p->ID = wall ? 2 : 1;
    p->IsFree = !wall;
    p->NoSlip = wall;
    p->Mass = 2.0 * (dx / 2.0) * 2.0 * (dx / 2.0) * rho;
    if (!wall) {
      p->Density = rho * std::pow((1 + 7.0 * g * (H - yb) / (cs * cs)), (1.0 / 7.0));
      p->Densityb = p->Density;
    }
  }
  if (argc > 4 && std::strcmp(argv[4], "user") == 0) {
    dom.OutputName[0] = "VelocityX";
    dom.OutputName[1] = "Density2";
    dom.OutputName[2] = "ShearRate";
    dom.UserOutput = &VelocityDensityOutput;
  }
  const double dt = 0.25 * h / cs;
  dom.Solve(/*tf*/ tf, /*dt*/ dt, /*dtOut*/ dtout, argv[1], 999);
  return 0;
}
MECHSYS_CATCH
