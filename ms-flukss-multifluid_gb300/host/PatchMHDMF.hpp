// PatchMHDMF.hpp - C++ host object with the configuration surface of the
// reference patch integrator (src/PatchMHDAM.H, srcIdeal/PatchMHDMF.H), built
// on the C ABI of include/mf_patch.h.  A caller that today configures a
// PatchMHDMF through its setters (main/MHDAM.cpp:771-1046) and calls
// updateState per patch (srcIdeal/AMRLevelIdealMHD.cpp:1248-1256) makes the
// same calls here, with device fabs instead of FArrayBox.
#pragma once

#include <stdexcept>
#include <string>

#include "../../include/mf_patch.h"

namespace mfgpu {

class PatchMHDMF {
 public:
  // PatchMHDAM::eTimeApproximation
  enum eTimeApproximation { TA_FirstOrder = 0, TA_Hancock = 1, TA_RK2 = 2 };

  // PatchMHDMF(int a_nFluids) (srcIdeal/PatchMHDMF.cpp:28-33)
  PatchMHDMF(int spaceDim, int nFluids);
  ~PatchMHDMF();
  PatchMHDMF(const PatchMHDMF&) = delete;
  PatchMHDMF& operator=(const PatchMHDMF&) = delete;

  // Riemann solver selection as RiemannSolver::make(iFlux, model, entropyFix)
  // (src/RiemannSolver.cpp:13-112); with GLM the solver is iFlux+100.
  void setRiemannSolver(int iFlux, double entropyFix = 0.3);
  // Reconstruction: minmod everywhere, then the per-variable limiters of the
  // plasma primitives (main/MHDAM.cpp:927-1009).
  void setReconstruction(const int limiters[8], bool checkPositivity);
  void setTimeApproximation(eTimeApproximation m);
  void setDivBMethod(int method);
  void set8waveFlag(int use8wave);
  // divB_cleaning = 5: GLM with Ch = factorCh*dx/dt, Cp = sqrt(Ch*dx/factorCp)
  void setDivergenceCleaning(int method, double factorCh = 1.0, double factorCp = 1.0);
  void setCurrentTime(double t);
  // EOS constants of /eos/ (gamma, smallr, smallp)
  void setEOS(double gamma, double smallr, double smallp);
  // Tracking surfaces: EqSysMHDMF(iDedner, nFluids, nTrackingSurfaces) and the
  // limiter of their slopes (main/MHDAM.cpp:709-718, 1005-1006).  regionTracer:
  // the last surface is the heliosphere's region tracer (region_tracer,
  // swlism/HeliosphericProblem.cpp:2538-2575) and lismU the interstellar flow
  // direction (lismUX/UY/UZ); null keeps the current one.
  void setTrackingSurfaces(int nSurfaces, int limiterLS, bool regionTracer = false,
                           const double* lismU = nullptr);
  // Problem domain in index space, periodicity and the uniform cell size.
  void define(const mf_box& domain, const int periodic[3], double dx);
  // Full parameter access for the physics options the setters do not cover
  // (charge exchange, regions, inner sphere, far-field boundary).
  mf_params& params() { return m_p; }

  int numGhostCells() const;
  int numStates() const { return mf_params_num_cons(&m_p); }
  void setCorrectionPotential(double ch, double cp);

  // PatchMHDAM::updateState (src/PatchMHDAM.H:252-260): U on the device with
  // numGhostCells() filled ghost layers; F (nullable, SpaceDim fabs) receives
  // the fluxes; divB (nullable) the divergence of B on the box.
  void updateState(mf_fab& U, mf_fab* F, double& newDt, int minDtCell[3], mf_fab* divB,
                   double dt, const mf_box& box, void* stream = nullptr);
  // The same with updateState's EdgeBox E (constrained transport: the step's
  // edge field as EdgeBox fabs on box, 3 in 3D, 1 nodal in 2D; may be null).
  void updateState(mf_fab& U, mf_fab* F, mf_fab* E, double& newDt, int minDtCell[3],
                   mf_fab* divB, double dt, const mf_box& box, void* stream = nullptr);
  // PatchMHDMF::recalculateMagneticField (srcIdeal/PatchMHDMF.cpp:1461-1484)
  void recalculateMagneticField(mf_fab& U, const mf_fab& Uold, const mf_fab* E, double dt,
                                const mf_box& box, void* stream = nullptr);
  // PatchMHDMF::computeDt (srcIdeal/PatchMHDMF.cpp:66-146)
  double computeDt(const mf_fab& U, const mf_box& box, int minDtCell[3],
                   void* stream = nullptr);

  mf_ctx* context();

 private:
  void invalidate();
  mf_params m_p;
  mf_ctx* m_ctx = nullptr;
  double m_time = 0.0;
};

class MFError : public std::runtime_error {
 public:
  MFError(mf_status s, const std::string& what)
      : std::runtime_error(what + ": " + mf_status_string(s)), status(s) {}
  mf_status status;
};

}  // namespace mfgpu
