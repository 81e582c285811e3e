/*
 * Instrumented driver for the UNMODIFIED reference (TEST INFRASTRUCTURE ONLY).
 *
 * Built by oracle/build_ref.sh against the reference's own Source/ and
 * External/ headers plus the project-written shims in oracle/shim/, into
 * oracle/_ref/ref_driver. It never ships and nothing in the product calls it.
 *
 * Modes
 *   box  <out> dim tag Vx Vy Vz Lx Ly Lz r rho h type rot random fixed
 *        Domain::AddBoxLength (Source/Domain.cpp:294-495); dumps x, mass,
 *        density, h of the generated particles.
 *   run  <in> <out> nsteps nproc [dump_step ...]
 *        Builds a Domain from the state directory <in>, performs Solve's
 *        set-up (Source/Domain.cpp:1746-1749) and then its per-step body
 *        (Source/Domain.cpp:1764-1792) nsteps times, with output disabled.
 *        After each listed step k it writes the full particle state to
 *        <out>/step_<k>/, and the pair lists MainNeighbourSearch produced
 *        from that state (first step after k) to <out>/pairs_<k>/.
 *        Per-phase wall times are printed as one JSON line.
 *
 * Private Domain members (time, time step, set-up checks) are reached through
 * pointers-to-member obtained by explicit template instantiation, which C++
 * permits to name private members; no reference source is edited. A constant body force (config key body_force) is applied through the
 * GeneralBefore hook exactly like the UserAcc hook of 1-Poiseuille.cpp:23-29.
 */
#include "Domain.h"

#include <omp.h>
#include <sys/stat.h>

#include <chrono>
#include <set>
#include <string>
#include <vector>

#include "state_io.h"

/* Private-member access: an explicit instantiation may name private members
 * ([temp.spec]/6); the friend function hands the pointer-to-member out. */
template <typename Tag, typename Tag::type M>
struct PsphRob {
  friend typename Tag::type psph_get(Tag) { return M; }
};
#define PSPH_ROB(TAGNAME, TYPE, MEMBER)          \
  struct TAGNAME {                               \
    using type = TYPE;                           \
    friend type psph_get(TAGNAME);               \
  };                                             \
  template struct PsphRob<TAGNAME, &SPH::Domain::MEMBER>;
PSPH_ROB(RobTime, double SPH::Domain::*, Time)
PSPH_ROB(RobDeltat, double SPH::Domain::*, deltat)
PSPH_ROB(RobDeltatmin, double SPH::Domain::*, deltatmin)
PSPH_ROB(RobDeltatint, double SPH::Domain::*, deltatint)
PSPH_ROB(RobCellfac, double SPH::Domain::*, Cellfac)
PSPH_ROB(RobInitialChecks, void (SPH::Domain::*)(), InitialChecks)
PSPH_ROB(RobAdaptive, void (SPH::Domain::*)(), AdaptiveTimeStep)
#define DOM_TIME(d) ((d).*psph_get(RobTime()))
#define DOM_DT(d) ((d).*psph_get(RobDeltat()))
#define DOM_DTMIN(d) ((d).*psph_get(RobDeltatmin()))
#define DOM_DTINT(d) ((d).*psph_get(RobDeltatint()))
#define DOM_CELLFAC(d) ((d).*psph_get(RobCellfac()))

static double g_body_force[3] = {0.0, 0.0, 0.0};

static void BodyForceHook(SPH::Domain& dom) {
  Vec3_t bf(g_body_force[0], g_body_force[1], g_body_force[2]);
#pragma omp parallel for schedule(static) num_threads(dom.Nproc)
  for (size_t i = 0; i < dom.Particles.Size(); i++)
    if (dom.Particles[i]->IsFree) dom.Particles[i]->a += bf;
}

/* In/out-flow profiles written the way the reference's drivers write their
 * InCon / OutCon hooks (Old_Tests/HydraulicJump.cpp:29-53): a hydrostatic
 * density under a level and a velocity that varies across the channel.
 * Config key flow_profile = H cs g (channel height, sound speed, gravity). */
static double g_prof[3] = {0.0, 0.0, 0.0};

static void ProfileInCon(Vec3_t& position, Vec3_t& Vel, double& Den, SPH::Boundary& bdry) {
  const double H = g_prof[0], Cs = g_prof[1], G = g_prof[2];
  const double y = position(1);
  Vel = bdry.inv(0) * 4.0 * y * (H - y) / (H * H), 0.0, 0.0;
  Den = bdry.inDensity * pow((1.0 + 7.0 * G * (H - y) / (Cs * Cs)), 1.0 / 7.0);
}

static void ProfileOutCon(Vec3_t& position, Vec3_t& Vel, double& Den, SPH::Boundary& bdry) {
  const double H = g_prof[0], Cs = g_prof[1], G = g_prof[2];
  const double y = position(1);
  Vel = bdry.outv(0) * (0.5 + y / H), 0.0, 0.0;
  Den = bdry.outDensity * pow((1.0 + 7.0 * G * (0.5 * H - y) / (Cs * Cs)), 1.0 / 7.0);
  if (y > 0.5 * H) Den = bdry.outDensity;
}

/* A GeneralAfter hook written the way the reference's soil drivers write their
 * UserDamping (Old_Tests/Embankment.cpp:31-58): while Time < t_end the free
 * particles of one material are damped (a -= DampS v), and once Time reaches
 * t_change the particles with one tag get a new cohesion and friction angle.
 * Config key damping = DampS t_end material t_change tag cohesion phi. */
static double g_damp[7] = {0, 0, 0, 0, 0, 0, 0};
static int g_damp_check = 0;

static void DampingHook(SPH::Domain& dom) {
  const double t = DOM_TIME(dom);
  if (t < g_damp[1])
    for (size_t i = 0; i < dom.Particles.Size(); i++)
      if (dom.Particles[i]->IsFree && dom.Particles[i]->Material == (int)g_damp[2])
        dom.Particles[i]->a -= g_damp[0] * dom.Particles[i]->v;
  if (t >= g_damp[3] && g_damp_check == 0) {
    for (size_t i = 0; i < dom.Particles.Size(); i++)
      if (dom.Particles[i]->ID == (int)g_damp[4] && dom.Particles[i]->Material == (int)g_damp[2]) {
        dom.Particles[i]->c = g_damp[5];
        dom.Particles[i]->phi = g_damp[6];
      }
    g_damp_check = 1;
  }
}

/* A GeneralBefore hook that adds a position-dependent acceleration to the
 * free particles (a spring towards a point). Config key spring = k xc yc. */
static double g_spring[3] = {0, 0, 0};

static void SpringHook(SPH::Domain& dom) {
  for (size_t i = 0; i < dom.Particles.Size(); i++)
    if (dom.Particles[i]->IsFree) {
      dom.Particles[i]->a(0) += g_spring[0] * (g_spring[1] - dom.Particles[i]->x(0));
      dom.Particles[i]->a(1) += g_spring[0] * (g_spring[2] - dom.Particles[i]->x(1));
    }
}

static void mkdir_p(const std::string& d) { mkdir(d.c_str(), 0755); }

static void cfg_line(FILE* f, const char* k, const double* v, int n) {
  fprintf(f, "%s", k);
  for (int i = 0; i < n; ++i) fprintf(f, " %.17g", v[i]);
  fprintf(f, "\n");
}

static int load_state(SPH::Domain& dom, const char* dir) {
  double v[3];
  int n = (int)psph_io_cfg1(dir, "n", -1);
  if (n < 0) return -1;
  dom.Dimension = (int)psph_io_cfg1(dir, "dimension", 2);
  dom.Kernel_Set((Kernels_Type)(int)psph_io_cfg1(dir, "kernel_type", 0));
  dom.Viscosity_Eq_Set((Viscosity_Eq_Type)(int)psph_io_cfg1(dir, "vis_eq", 0));
  dom.Gradient_Approach_Set((Gradient_Type)(int)psph_io_cfg1(dir, "gradient_type", 0));
  dom.Scheme = (size_t)psph_io_cfg1(dir, "scheme", 0);
  dom.XSPH = psph_io_cfg1(dir, "xsph", 0.0);
  dom.sqrt_h_a = psph_io_cfg1(dir, "sqrt_h_a", 0.0025);
  dom.R = psph_io_cfg1(dir, "R", 0.0);
  dom.InitialDist = psph_io_cfg1(dir, "initial_dist", 0.0);
  if (psph_io_cfg(dir, "periodic", v, 3) == 3)
    for (int d = 0; d < 3; ++d) dom.BC.Periodic[d] = v[d] != 0.0;
  if (psph_io_cfg(dir, "gravity", v, 3) == 3) dom.Gravity = v[0], v[1], v[2];
  if (psph_io_cfg(dir, "dom_max", v, 3) == 3) dom.DomMax = v[0], v[1], v[2];
  if (psph_io_cfg(dir, "dom_min", v, 3) == 3) dom.DomMin = v[0], v[1], v[2];
  if (psph_io_cfg(dir, "body_force", v, 3) == 3) {
    for (int d = 0; d < 3; ++d) g_body_force[d] = v[d];
    if (v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0) dom.GeneralBefore = &BodyForceHook;
  }
  dom.SWIType = (size_t)psph_io_cfg1(dir, "swi_type", 0);
  dom.FSI = psph_io_cfg1(dir, "fsi", 0) != 0.0;
  dom.BC.InOutFlow = (int)psph_io_cfg1(dir, "in_out_flow", 0);
  dom.BC.MassConservation = psph_io_cfg1(dir, "mass_conservation", 0) != 0.0;
  if (psph_io_cfg1(dir, "bc_cellfac", 0.0) > 0.0) dom.BC.cellfac = psph_io_cfg1(dir, "bc_cellfac", 0.0);
  if (psph_io_cfg(dir, "in_v", v, 3) == 3) dom.BC.inv = v[0], v[1], v[2];
  if (psph_io_cfg(dir, "out_v", v, 3) == 3) dom.BC.outv = v[0], v[1], v[2];
  dom.BC.inDensity = psph_io_cfg1(dir, "in_density", 0.0);
  dom.BC.outDensity = psph_io_cfg1(dir, "out_density", 0.0);
  if (psph_io_cfg(dir, "damping", g_damp, 7) == 7) dom.GeneralAfter = &DampingHook;
  if (psph_io_cfg(dir, "spring", g_spring, 3) == 3) dom.GeneralBefore = &SpringHook;
  if (psph_io_cfg(dir, "flow_profile", g_prof, 3) == 3) {
    dom.InCon = &ProfileInCon;
    dom.OutCon = &ProfileOutCon;
  }
  dom.MuMax = 0.0;  // left uninitialised by the Domain constructor
  dom.CsMax = 0.0;

  std::vector<int32_t> ibuf(n);
  std::vector<double> dbuf(n), vbuf(3 * (size_t)n), tbuf(9 * (size_t)n);
#define RD(name, buf, bytes) psph_io_read(dir, name, buf, bytes)
  if (RD("x", vbuf.data(), 24 * (size_t)n)) return -2;
  for (int i = 0; i < n; ++i)
    dom.AddSingleParticle(0, Vec3_t(vbuf[3 * i], vbuf[3 * i + 1], vbuf[3 * i + 2]), 0.0, 1.0, 1.0, false);

#define SET_INT(NAME, EXPR)                                  \
  if (RD(#NAME, ibuf.data(), 4 * (size_t)n) == 0)            \
    for (int i = 0; i < n; ++i) {                            \
      SPH::Particle* P = dom.Particles[i];                   \
      int32_t val = ibuf[i];                                 \
      EXPR;                                                  \
    }
  SET_INT(id, P->ID = val)
  SET_INT(material, P->Material = val)
  SET_INT(is_free, P->IsFree = val != 0)
  SET_INT(no_slip, P->NoSlip = val != 0)
  SET_INT(pres_eq, P->PresEq = (size_t)val)
  SET_INT(shepard, P->Shepard = val != 0)
  SET_INT(les, P->LES = val != 0)
  SET_INT(vis_m, P->VisM = (size_t)val)
  SET_INT(fail, P->Fail = (size_t)val)
  SET_INT(seepage_type, P->SeepageType = (size_t)val)
  SET_INT(var_porosity, P->VarPorosity = val != 0)
  SET_INT(is_sat, P->IsSat = val != 0)
  SET_INT(in_out, P->InOut = (size_t)val)
#define SET_F64(NAME, MEMBER)                                           \
  if (RD(#NAME, dbuf.data(), 8 * (size_t)n) == 0)                       \
    for (int i = 0; i < n; ++i) dom.Particles[i]->MEMBER = dbuf[i];
  SET_F64(density, Density) SET_F64(densitya, Densitya) SET_F64(densityb, Densityb)
  SET_F64(ddensity, dDensity) SET_F64(pressure, Pressure) SET_F64(mass, Mass) SET_F64(h, h)
  SET_F64(cs, Cs) SET_F64(p0, P0) SET_F64(ref_density, RefDensity) SET_F64(fpmassc, FPMassC)
  SET_F64(alpha, Alpha) SET_F64(beta, Beta) SET_F64(mu, Mu) SET_F64(mu_ref, MuRef) SET_F64(t0, T0)
  SET_F64(bingham_m, m) SET_F64(csmag, CSmag) SET_F64(ti, TI) SET_F64(tin, TIn)
  SET_F64(ti_init_dist, TIInitDist) SET_F64(g_mod, G) SET_F64(k_mod, K) SET_F64(sigmay, Sigmay)
  SET_F64(cohesion, c) SET_F64(phi, phi) SET_F64(psi, psi) SET_F64(zwab, ZWab)
  SET_F64(sumden, SumDen) SET_F64(sumkernel, SumKernel) SET_F64(shear_rate, ShearRate)
  SET_F64(sbar, SBar) SET_F64(n0, n0) SET_F64(k, k) SET_F64(k2, k2) SET_F64(d, d) SET_F64(rho_f, RhoF)
  SET_F64(s, S)
#define SET_VEC(NAME, MEMBER)                                                         \
  if (RD(#NAME, vbuf.data(), 24 * (size_t)n) == 0)                                    \
    for (int i = 0; i < n; ++i)                                                       \
      dom.Particles[i]->MEMBER = vbuf[3 * i], vbuf[3 * i + 1], vbuf[3 * i + 2];
  SET_VEC(v, v) SET_VEC(va, va) SET_VEC(vb, vb) SET_VEC(a, a) SET_VEC(nsv, NSv) SET_VEC(vxsph, VXSPH)
#define SET_TEN(NAME, MEMBER)                                                   \
  if (RD(#NAME, tbuf.data(), 72 * (size_t)n) == 0)                              \
    for (int i = 0; i < n; ++i)                                                 \
      for (int r = 0; r < 3; ++r)                                               \
        for (int c = 0; c < 3; ++c) dom.Particles[i]->MEMBER(r, c) = tbuf[9 * i + 3 * r + c];
  SET_TEN(sigma, Sigma) SET_TEN(sigmaa, Sigmaa) SET_TEN(sigmab, Sigmab)
  SET_TEN(shear_stress, ShearStress) SET_TEN(shear_stressa, ShearStressa)
  SET_TEN(shear_stressb, ShearStressb) SET_TEN(strain, Strain) SET_TEN(straina, Straina)
  SET_TEN(strainb, Strainb) SET_TEN(strain_rate, StrainRate) SET_TEN(rotation_rate, RotationRate)
  SET_TEN(tir, TIR)
  // mass-derived volume, as the Particle constructor computes it, unless given
  for (int i = 0; i < n; ++i) dom.Particles[i]->V = dom.Particles[i]->Mass / dom.Particles[i]->RefDensity;
  SET_F64(volume, V)
  double ss = psph_io_cfg1(dir, "shepard_step", 40);
  for (int i = 0; i < n; ++i) dom.Particles[i]->ShepardStep = (size_t)ss;
  return n;
}

static void dump_state(SPH::Domain& dom, const std::string& dir, long step) {
  mkdir_p(dir);
  size_t n = dom.Particles.Size();
  std::vector<int32_t> ib(n);
  std::vector<double> db(n), vb(3 * n), tb(9 * n);
  const char* d = dir.c_str();
#define W_INT(NAME, EXPR)                                                  \
  for (size_t i = 0; i < n; ++i) { SPH::Particle* P = dom.Particles[i]; ib[i] = (int32_t)(EXPR); } \
  psph_io_write(d, #NAME, ib.data(), 4 * n);
  W_INT(id, P->ID) W_INT(material, P->Material) W_INT(is_free, P->IsFree) W_INT(no_slip, P->NoSlip)
  W_INT(pres_eq, P->PresEq) W_INT(shepard, P->Shepard) W_INT(les, P->LES) W_INT(vis_m, P->VisM)
  W_INT(fail, P->Fail) W_INT(seepage_type, P->SeepageType) W_INT(var_porosity, P->VarPorosity)
  W_INT(is_sat, P->IsSat) W_INT(in_out, P->InOut)
#define W_F64(NAME, MEMBER)                                           \
  for (size_t i = 0; i < n; ++i) db[i] = dom.Particles[i]->MEMBER;    \
  psph_io_write(d, #NAME, db.data(), 8 * n);
  W_F64(density, Density) W_F64(densitya, Densitya) W_F64(densityb, Densityb)
  W_F64(ddensity, dDensity) W_F64(pressure, Pressure) W_F64(mass, Mass) W_F64(h, h) W_F64(cs, Cs)
  W_F64(p0, P0) W_F64(ref_density, RefDensity) W_F64(fpmassc, FPMassC) W_F64(alpha, Alpha)
  W_F64(beta, Beta) W_F64(mu, Mu) W_F64(mu_ref, MuRef) W_F64(t0, T0) W_F64(bingham_m, m)
  W_F64(csmag, CSmag) W_F64(ti, TI) W_F64(tin, TIn) W_F64(ti_init_dist, TIInitDist) W_F64(g_mod, G)
  W_F64(k_mod, K) W_F64(sigmay, Sigmay) W_F64(cohesion, c) W_F64(phi, phi) W_F64(psi, psi)
  W_F64(zwab, ZWab) W_F64(sumden, SumDen) W_F64(sumkernel, SumKernel) W_F64(shear_rate, ShearRate)
  W_F64(sbar, SBar) W_F64(n0, n0) W_F64(k, k) W_F64(k2, k2) W_F64(d, d) W_F64(rho_f, RhoF)
  W_F64(volume, V) W_F64(s, S)
#define W_VEC(NAME, MEMBER)                                                       \
  for (size_t i = 0; i < n; ++i)                                                  \
    for (int k = 0; k < 3; ++k) vb[3 * i + k] = dom.Particles[i]->MEMBER(k);      \
  psph_io_write(d, #NAME, vb.data(), 24 * n);
  W_VEC(x, x) W_VEC(v, v) W_VEC(va, va) W_VEC(vb, vb) W_VEC(a, a) W_VEC(nsv, NSv) W_VEC(vxsph, VXSPH)
#define W_TEN(NAME, MEMBER)                                                              \
  for (size_t i = 0; i < n; ++i)                                                         \
    for (int r = 0; r < 3; ++r)                                                          \
      for (int c = 0; c < 3; ++c) tb[9 * i + 3 * r + c] = dom.Particles[i]->MEMBER(r, c); \
  psph_io_write(d, #NAME, tb.data(), 72 * n);
  W_TEN(sigma, Sigma) W_TEN(sigmaa, Sigmaa) W_TEN(sigmab, Sigmab) W_TEN(shear_stress, ShearStress)
  W_TEN(shear_stressa, ShearStressa) W_TEN(shear_stressb, ShearStressb) W_TEN(strain, Strain)
  W_TEN(straina, Straina) W_TEN(strainb, Strainb) W_TEN(strain_rate, StrainRate)
  W_TEN(rotation_rate, RotationRate) W_TEN(tir, TIR)

  FILE* f = fopen((dir + "/config.txt").c_str(), "w");
  double t[3];
  t[0] = (double)n;
  cfg_line(f, "n", t, 1);
  t[0] = (double)step;
  cfg_line(f, "step", t, 1);
  cfg_line(f, "time", &DOM_TIME(dom), 1);
  cfg_line(f, "deltat", &DOM_DT(dom), 1);
  cfg_line(f, "deltatmin", &DOM_DTMIN(dom), 1);
  cfg_line(f, "deltatint", &DOM_DTINT(dom), 1);
  cfg_line(f, "blpf", dom.BLPF.data(), 3);
  cfg_line(f, "trpr", dom.TRPR.data(), 3);
  cfg_line(f, "cell_size", dom.CellSize.data(), 3);
  for (int k = 0; k < 3; ++k) t[k] = dom.CellNo[k];
  cfg_line(f, "cell_no", t, 3);
  cfg_line(f, "dom_size", dom.DomSize.data(), 3);
  cfg_line(f, "hmax", &dom.hmax, 1);
  cfg_line(f, "rhomax", &dom.rhomax, 1);
  cfg_line(f, "cellfac", &DOM_CELLFAC(dom), 1);
  size_t first_free = 0;
  while (first_free < n && !dom.Particles[first_free]->IsFree) ++first_free;
  if (first_free < n) {
    SPH::Particle* P = dom.Particles[first_free];
    t[0] = P->FirstStep;
    cfg_line(f, "first_step", t, 1);
    t[0] = P->ct;
    cfg_line(f, "ct", t, 1);
    t[0] = (double)P->ShepardCounter;
    cfg_line(f, "shepard_counter", t, 1);
  }
  fclose(f);
  // per-particle cell indices (CC) for the cell-list checks
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) vb[3 * i + k] = dom.Particles[i]->CC[k];
  psph_io_write(d, "cc", vb.data(), 24 * n);
}

static void dump_pairs(SPH::Domain& dom, const std::string& dir) {
  mkdir_p(dir);
  const char* names[3] = {"sm", "fsm", "nsm"};
  Array<Array<std::pair<size_t, size_t> > >* lists[3] = {&dom.SMPairs, &dom.FSMPairs, &dom.NSMPairs};
  for (int l = 0; l < 3; ++l) {
    std::vector<int64_t> buf;
    for (size_t t = 0; t < lists[l]->Size(); ++t)
      for (size_t k = 0; k < (*lists[l])[t].Size(); ++k) {
        buf.push_back((int64_t)(*lists[l])[t][k].first);
        buf.push_back((int64_t)(*lists[l])[t][k].second);
      }
    psph_io_write(dir.c_str(), names[l], buf.data(), buf.size() * 8);
  }
}

typedef std::chrono::steady_clock clk;
static double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

static int run(const char* in, const char* out, long nsteps, int nproc, const std::set<long>& dumps) {
  SPH::Domain dom;
  dom.Nproc = nproc;
  if (load_state(dom, in) < 0) {
    fprintf(stderr, "cannot read state %s\n", in);
    return 2;
  }
  double dt = psph_io_cfg1(in, "dt", 0.0);
  DOM_DT(dom) = DOM_DTINT(dom) = DOM_DTMIN(dom) = dt;  // Source/Domain.cpp:1743
  DOM_TIME(dom) = psph_io_cfg1(in, "time", 0.0);
  mkdir_p(out);
  // Solve's set-up (Source/Domain.cpp:1746-1751), without the log file/output
  (dom.*psph_get(RobInitialChecks()))();
  dom.CellInitiate();
  dom.ListGenerate();
  dom.WholeVelocity();
  double t_phase[7] = {0, 0, 0, 0, 0, 0, 0};  // start, search, primary, last, move, relist, total
  if (dumps.count(0)) dump_state(dom, std::string(out) + "/step_0", 0);
  clk::time_point t_all = clk::now();
  for (long s = 0; s < nsteps; ++s) {
    // Solve's per-step body (Source/Domain.cpp:1764-1792), output disabled
    clk::time_point t0 = clk::now();
    dom.StartAcceleration(dom.Gravity);
    if (dom.BC.InOutFlow > 0) dom.InFlowBCFresh();
    clk::time_point t1 = clk::now();
    dom.MainNeighbourSearch();
    clk::time_point t2 = clk::now();
    if (dumps.count(s)) dump_pairs(dom, std::string(out) + "/pairs_" + std::to_string(s));
    clk::time_point t2b = clk::now();
    dom.GeneralBefore(dom);
    dom.PrimaryComputeAcceleration();
    clk::time_point t3 = clk::now();
    dom.LastComputeAcceleration();
    dom.GeneralAfter(dom);
    clk::time_point t4 = clk::now();
    (dom.*psph_get(RobAdaptive()))();
    dom.Move(DOM_DT(dom));
    DOM_TIME(dom) += DOM_DT(dom);
    clk::time_point t5 = clk::now();
    if (dom.BC.InOutFlow > 0) dom.InFlowBCLeave(); else dom.CheckParticleLeave();
    dom.CellReset();
    dom.ListGenerate();
    clk::time_point t6 = clk::now();
    t_phase[0] += secs(t0, t1);
    t_phase[1] += secs(t1, t2);
    t_phase[2] += secs(t2b, t3);
    t_phase[3] += secs(t3, t4);
    t_phase[4] += secs(t4, t5);
    t_phase[5] += secs(t5, t6);
    if (dumps.count(s + 1)) {
      clk::time_point d0 = clk::now();
      dump_state(dom, std::string(out) + "/step_" + std::to_string(s + 1), s + 1);
      t_all += clk::now() - d0;  // exclude dump time from the total
    }
  }
  t_phase[6] = secs(t_all, clk::now());
  printf("{\"steps\": %ld, \"nproc\": %d, \"n\": %zu, \"start_s\": %.6f, \"search_s\": %.6f, "
         "\"primary_s\": %.6f, \"last_s\": %.6f, \"move_s\": %.6f, \"relist_s\": %.6f, \"total_s\": %.6f}\n",
         nsteps, nproc, dom.Particles.Size(), t_phase[0], t_phase[1], t_phase[2], t_phase[3], t_phase[4],
         t_phase[5], t_phase[6]);
  return 0;
}

static int box(int argc, char** argv) {
  if (argc < 18) return 2;
  SPH::Domain dom;
  dom.Dimension = atoi(argv[3]);
  int tag = atoi(argv[4]);
  Vec3_t V(atof(argv[5]), atof(argv[6]), atof(argv[7]));
  dom.AddBoxLength(tag, V, atof(argv[8]), atof(argv[9]), atof(argv[10]), atof(argv[11]), atof(argv[12]),
                   atof(argv[13]), atoi(argv[14]), atoi(argv[15]), atoi(argv[16]) != 0, atoi(argv[17]) != 0);
  std::string out = argv[2];
  mkdir_p(out);
  size_t n = dom.Particles.Size();
  std::vector<double> x(3 * n), m(n), rho(n), h(n);
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) x[3 * i + k] = dom.Particles[i]->x(k);
    m[i] = dom.Particles[i]->Mass;
    rho[i] = dom.Particles[i]->Density;
    h[i] = dom.Particles[i]->h;
  }
  psph_io_write(out.c_str(), "x", x.data(), 24 * n);
  psph_io_write(out.c_str(), "mass", m.data(), 8 * n);
  psph_io_write(out.c_str(), "density", rho.data(), 8 * n);
  psph_io_write(out.c_str(), "h", h.data(), 8 * n);
  FILE* f = fopen((out + "/config.txt").c_str(), "w");
  fprintf(f, "n %zu\nR %.17g\n", n, dom.R);
  fclose(f);
  return 0;
}

int main(int argc, char** argv) try {
  if (argc >= 2 && std::string(argv[1]) == "box") return box(argc, argv);
  if (argc >= 6 && std::string(argv[1]) == "run") {
    std::set<long> dumps;
    for (int i = 6; i < argc; ++i) dumps.insert(atol(argv[i]));
    return run(argv[2], argv[3], atol(argv[4]), atoi(argv[5]), dumps);
  }
  fprintf(stderr, "usage: ref_driver box|run ...\n");
  return 2;
}
MECHSYS_CATCH
