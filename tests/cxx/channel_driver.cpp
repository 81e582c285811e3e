// A driver in the reference's style for an in/out-flow channel (the
// Old_Tests/HydraulicJump.cpp pattern: user InCon / OutCon / AllCon hooks,
// BC.InOutFlow = 3, MassConservation), built against
// include/persiansph/Domain.h. The channel is the channel_profile case of
// tests/golden/cases.py, started by WholeVelocity from the in-flow profile and
// solved to tf; the final state is written as raw binary: int64 n, x[3n],
// v[3n], density[n], pressure[n], double time, int32 InOut[n], int32 ID[n].
#include <cstdio>
#include <cstdlib>

#include "Domain.h"

static double H = 0.1, Cs = 20.0;
static const double G = 9.81;

void UserInFlowCon(Vec3_t& position, Vec3_t& Vel, double& Den, SPH::Boundary& bdry) {
  const double y = position(1);
  Vel = bdry.inv(0) * 4.0 * y * (H - y) / (H * H), 0.0, 0.0;
  Den = bdry.inDensity * pow((1.0 + 7.0 * G * (H - y) / (Cs * Cs)), 1.0 / 7.0);
}

void UserOutFlowCon(Vec3_t& position, Vec3_t& Vel, double& Den, SPH::Boundary& bdry) {
  const double y = position(1);
  Vel = bdry.outv(0) * (0.5 + y / H), 0.0, 0.0;
  Den = bdry.outDensity * pow((1.0 + 7.0 * G * (0.5 * H - y) / (Cs * Cs)), 1.0 / 7.0);
  if (y > 0.5 * H) Den = bdry.outDensity;
}

int main(int argc, char** argv) try {
  if (argc < 3) {
    std::printf("usage: %s out.bin tf\n", argv[0]);
    return 2;
  }
  const double tf = std::atof(argv[2]);
  SPH::Domain dom;
  dom.Dimension = 2;
  dom.Nproc = 4;
  dom.Scheme = 0;
  dom.Kernel_Set(Qubic_Spline);
  dom.Viscosity_Eq_Set(Morris);
  dom.Gradient_Approach_Set(Squared_density);
  dom.Gravity = 0.0, 0.0, 0.0;

  const double dx = 0.01, L = 0.5, U = 2.0, rho = 1000.0, mu = 1.0e-3;
  const double h = 1.2 * dx;
  dom.InitialDist = dx;
  dom.AddBoxLength(1, Vec3_t(0.0, -3.0 * dx, 0.0), L + dx / 10.0, H + 2 * 3 * dx + dx / 10.0, 0, dx / 2.0, rho, h, 1,
                   0, false, false);
  for (size_t a = 0; a < dom.Particles.Size(); a++) {
    SPH::Particle* p = dom.Particles[a];
    const double yb = p->x(1);
    const bool wall = (yb < 0.0) || (yb > H);
    p->h = h;
    p->Density = rho;
    p->RefDensity = rho;
    p->Cs = Cs;
    p->PresEq = 1;
    p->Mu = mu;
    p->MuRef = mu;
    p->Material = 1;
    p->Alpha = 0.1;
    p->ID = wall ? 2 : 1;
    p->IsFree = !wall;
    p->NoSlip = wall;
    p->Mass = rho * dx * dx;
  }
  dom.BC.InOutFlow = 3;
  dom.BC.inv = U, 0.0, 0.0;
  dom.BC.inDensity = rho;
  dom.BC.outv = 2.0, 0.0, 0.0;
  dom.BC.outDensity = 1000.0;
  dom.BC.MassConservation = true;
  dom.BC.allv = U, 0.0, 0.0;
  dom.BC.allDensity = rho;
  dom.InCon = &UserInFlowCon;
  dom.OutCon = &UserOutFlowCon;
  dom.AllCon = &UserInFlowCon;
  const double dt = 0.25 * h / Cs;
  dom.Solve(/*tf*/ tf, /*dt*/ dt, /*dtOut*/ tf, nullptr, 999);

  FILE* f = std::fopen(argv[1], "wb");
  const int64_t n = (int64_t)dom.Particles.Size();
  std::fwrite(&n, sizeof n, 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(dom.Particles[a]->x.data(), sizeof(double), 3, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(dom.Particles[a]->v.data(), sizeof(double), 3, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(&dom.Particles[a]->Density, sizeof(double), 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(&dom.Particles[a]->Pressure, sizeof(double), 1, f);
  std::fwrite(&dom.Time, sizeof(double), 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) {
    const int32_t io = (int32_t)dom.Particles[a]->InOut;
    std::fwrite(&io, sizeof io, 1, f);
  }
  for (size_t a = 0; a < dom.Particles.Size(); a++) {
    const int32_t id = (int32_t)dom.Particles[a]->ID;
    std::fwrite(&id, sizeof id, 1, f);
  }
  std::fclose(f);
  return 0;
}
MECHSYS_CATCH
