// PatchMHDMF.cpp - configuration object over the C ABI (see PatchMHDMF.hpp).
#include "PatchMHDMF.hpp"

namespace mfgpu {

namespace {
void ok(mf_status s, const char* what) {
  if (s != MF_OK) throw MFError(s, what);
}
}  // namespace

PatchMHDMF::PatchMHDMF(int spaceDim, int nFluids) { mf_params_default(&m_p, spaceDim, nFluids); }

PatchMHDMF::~PatchMHDMF() { invalidate(); }

void PatchMHDMF::invalidate() {
  if (m_ctx) mf_destroy(m_ctx);
  m_ctx = nullptr;
}

void PatchMHDMF::setRiemannSolver(int iFlux, double entropyFix) {
  m_p.flux = iFlux;
  m_p.entropy_fix = entropyFix;
  invalidate();
}

void PatchMHDMF::setReconstruction(const int limiters[8], bool checkPositivity) {
  for (int v = 0; v < 8; ++v) m_p.limiter[v] = limiters[v];
  m_p.check_positivity = checkPositivity ? 1 : 0;
  invalidate();
}

void PatchMHDMF::setTrackingSurfaces(int nSurfaces, int limiterLS, bool regionTracer,
                                     const double* lismU) {
  m_p.num_tracking_surfaces = nSurfaces;
  m_p.limiter_ls = limiterLS;
  m_p.region_tracer = regionTracer ? 1 : 0;
  if (lismU)
    for (int d = 0; d < 3; ++d) m_p.lism_u[d] = lismU[d];
  invalidate();
}

void PatchMHDMF::setTimeApproximation(eTimeApproximation m) {
  m_p.time_approximation = (int)m;
  invalidate();
}

void PatchMHDMF::setDivBMethod(int method) {
  m_p.divb_method = method;
  invalidate();
}

void PatchMHDMF::set8waveFlag(int use8wave) {
  m_p.use_8wave = (use8wave == 1) ? 1 : 0;
  invalidate();
}

void PatchMHDMF::setDivergenceCleaning(int method, double factorCh, double factorCp) {
  m_p.divb_cleaning = method;
  m_p.factor_ch = factorCh;
  m_p.factor_cp = factorCp;
  invalidate();
}

void PatchMHDMF::setCurrentTime(double t) {
  m_time = t;
  if (m_ctx) ok(mf_set_current_time(m_ctx, t), "setCurrentTime");
}

void PatchMHDMF::setEOS(double gamma, double smallr, double smallp) {
  m_p.gamma = gamma;
  m_p.smallr = smallr;
  m_p.smallp = smallp;
  invalidate();
}

void PatchMHDMF::define(const mf_box& domain, const int periodic[3], double dx) {
  for (int d = 0; d < 3; ++d) {
    m_p.domain_lo[d] = domain.lo[d];
    m_p.domain_hi[d] = domain.hi[d];
    m_p.periodic[d] = periodic[d];
  }
  m_p.dx = dx;
  invalidate();
}

void PatchMHDMF::setCorrectionPotential(double ch, double cp) {
  m_p.dedner_ch = ch;
  m_p.dedner_cp = cp;
  if (m_ctx) ok(mf_set_dedner(m_ctx, ch, cp), "setCorrectionPotential");
}

int PatchMHDMF::numGhostCells() const {
  if (m_p.time_approximation == TA_RK2) return 4;
  if (m_p.time_approximation == TA_Hancock) return 3;
  return 2;
}

mf_ctx* PatchMHDMF::context() {
  if (!m_ctx) {
    ok(mf_create(&m_p, &m_ctx), "PatchMHDMF::define");
    ok(mf_set_current_time(m_ctx, m_time), "setCurrentTime");
  }
  return m_ctx;
}

void PatchMHDMF::updateState(mf_fab& U, mf_fab* F, double& newDt, int minDtCell[3],
                             mf_fab* divB, double dt, const mf_box& box, void* stream) {
  ok(mf_patch_update(context(), &U, &box, dt, F, divB, &newDt, minDtCell, stream),
     "PatchMHDMF::updateState");
}

void PatchMHDMF::updateState(mf_fab& U, mf_fab* F, mf_fab* E, double& newDt, int minDtCell[3],
                             mf_fab* divB, double dt, const mf_box& box, void* stream) {
  ok(mf_patch_update_e(context(), &U, &box, dt, F, divB, E, &newDt, minDtCell, stream),
     "PatchMHDMF::updateState");
}

void PatchMHDMF::recalculateMagneticField(mf_fab& U, const mf_fab& Uold, const mf_fab* E,
                                          double dt, const mf_box& box, void* stream) {
  ok(mf_recalculate_magnetic_field(context(), &U, &Uold, E, dt, &box, stream),
     "PatchMHDMF::recalculateMagneticField");
}

double PatchMHDMF::computeDt(const mf_fab& U, const mf_box& box, int minDtCell[3],
                             void* stream) {
  double dt = 0.0;
  ok(mf_compute_dt(context(), &U, &box, &dt, minDtCell, stream), "PatchMHDMF::computeDt");
  return dt;
}

}  // namespace mfgpu
