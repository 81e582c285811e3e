// A driver in the reference's style (the 3-DamBreak.cpp pattern), built
// against include/persiansph/Domain.h: the dam2d parity case of
// tests/golden/cases.py, solved to tf, final state written as raw binary:
// int64 n, x[3n], v[3n], density[n], pressure[n], double time.
// With a fourth argument "hooks" it also sets a GeneralBefore hook (a spring
// towards a point) and a GeneralAfter hook (damping of the fluid's
// accelerations for a while, then a new artificial viscosity for part of it).
#include <cstdio>
#include <cstdlib>
#include <string>

#include "Domain.h"

void UserSpring(SPH::Domain& dom) {
  for (size_t i = 0; i < dom.Particles.Size(); i++)
    if (dom.Particles[i]->IsFree) {
      dom.Particles[i]->a(0) += 20.0 * (0.5 - dom.Particles[i]->x(0));
      dom.Particles[i]->a(1) += 20.0 * (0.3 - dom.Particles[i]->x(1));
    }
}

void UserDamping(SPH::Domain& dom) {
  if (dom.Time < 0.02)
    for (size_t i = 0; i < dom.Particles.Size(); i++)
      if (dom.Particles[i]->IsFree) dom.Particles[i]->a -= 2.0 * dom.Particles[i]->v;
  if (dom.Time >= 0.01)
    for (size_t i = 0; i < dom.Particles.Size(); i++)
      if (dom.Particles[i]->IsFree && dom.Particles[i]->x(0) < 0.2) dom.Particles[i]->Alpha = 0.05;
}

int main(int argc, char** argv) try {
  if (argc < 3) {
    std::printf("usage: %s out.bin tf [precision]\n", argv[0]);
    return 2;
  }
  const double tf = std::atof(argv[2]);
  SPH::Domain dom;
  dom.Dimension = 2;
  dom.Nproc = 4;
  dom.Scheme = 0;
  dom.Viscosity_Eq_Set(Morris);
  dom.Kernel_Set(Qubic_Spline);
  dom.Gradient_Approach_Set(Squared_density);
  if (argc > 3) dom.Precision = std::atoi(argv[3]);

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
  if (argc > 4 && std::string(argv[4]) == "hooks") {
    dom.GeneralBefore = &UserSpring;
    dom.GeneralAfter = &UserDamping;
  }
  const double dt = 0.25 * h / cs;
  dom.Solve(/*tf*/ tf, /*dt*/ dt, /*dtOut*/ tf, nullptr, 999);

  FILE* f = std::fopen(argv[1], "wb");
  const int64_t n = (int64_t)dom.Particles.Size();
  std::fwrite(&n, sizeof n, 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(dom.Particles[a]->x.data(), sizeof(double), 3, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(dom.Particles[a]->v.data(), sizeof(double), 3, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(&dom.Particles[a]->Density, sizeof(double), 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(&dom.Particles[a]->Pressure, sizeof(double), 1, f);
  std::fwrite(&dom.Time, sizeof(double), 1, f);
  std::fclose(f);
  return 0;
}
MECHSYS_CATCH
