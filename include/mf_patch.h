/*
 * mf_patch.h - C ABI of the GB300 multi-fluid MHD patch integrator.
 *
 * The entry points replace the per-patch Godunov update of MHDAM / MS-FLUKSS
 * (MHDAM-3.2.4).  Every pointer that names state (mf_fab::data, face fluxes,
 * divB) is a DEVICE pointer unless the function name ends in _host.  No
 * function aborts; every call returns an mf_status.  There are no globals:
 * all physical and numerical parameters travel in mf_params, so runs with
 * different parameters can share one GPU.
 *
 * Reference interfaces replaced (paths inside the MHDAM-3.2.4 tree):
 *   mf_create / mf_destroy     the PatchMHDMF object set up by the driver
 *                              (main/MHDAM.cpp:771-1046) and cloned per level
 *                              (srcIdeal/PatchMHDMF.cpp:43-62).  The Fortran
 *                              COMMON blocks /eos/ (srcIdeal/EosCommon.fh:39-40),
 *                              /RiemSol/ (src/RSCommon.fh:6), /chargeexcm/
 *                              (srcIdeal/ChargeExchange.fh:8-10) and /Dedner/
 *                              become fields of mf_params.
 *   mf_num_ghost               PatchMHDAM::numGhostCells (src/PatchMHDAM.cpp:280-286)
 *   mf_set_current_time        PatchMHDAM::setCurrentTime (src/PatchMHDAM.cpp:272-276)
 *   mf_set_dedner              EqSysMHDMF::setCorrectionPotential -> SETDEDNERCONST
 *                              (src/DednerF.ChF:4-13)
 *   mf_patch_update(_e)        PatchMHDAM::updateState (src/PatchMHDAM.H:252-260,
 *                              src/PatchMHDAM.cpp:1192-1317); _e with its EdgeBox E
 *   mf_recalculate_magnetic_field
 *                              PatchMHDMF::recalculateMagneticField
 *                              (srcIdeal/PatchMHDMF.cpp:1461-1484)
 *   mf_compute_dt              PatchMHDMF::computeDt (srcIdeal/PatchMHDMF.cpp:66-146)
 *   mf_level_*                 AMRLevelIdealMHD::advance/step over all patches of a
 *                              level: ghost exchange (srcIdeal/AMRLevelIdealMHD.cpp:772),
 *                              the patch loop (:1203-1309) and the dt MIN
 *                              reduction (:1517-1529) with the GLM Ch/Cp update
 *                              (:1531-1548).
 *   mf_hier_*                  a subcycled hierarchy of levels: AMR_MHDAM::timeStep
 *                              (srcIdeal/AMR_MHDAM.cpp:1707-1880) with the coarse-fine
 *                              ghost interpolation PiecewiseLinearFillPatchMHDAM::fillInterp
 *                              (srcIdeal/PiecewiseLinearFillPatchMHDAM.cpp:382-900,
 *                              called at srcIdeal/AMRLevelIdealMHD.cpp:748-752), the
 *                              LevelFluxRegister increments and reflux (:1276-1308,
 *                              :1633-1642) and CoarseAverageExt::averageToCoarse (:1646,
 *                              src/CoarseAverageExt.cpp:117-192).
 *
 * Data layout (Chombo FArrayBox): one contiguous FP64 array per patch covering
 * the valid box grown by mf_num_ghost() cells on every side, component-major,
 * x fastest: data[((c*nz + (k-lo2))*ny + (j-lo1))*nx + (i-lo0)].  In 2D the
 * third index range is lo[2] = hi[2] = 0.
 */
#ifndef MF_PATCH_H
#define MF_PATCH_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mf_status {
  MF_OK = 0,
  MF_ERR_BAD_ARG = 1,      /* invalid argument (sizes, boxes, null pointers) */
  MF_ERR_OOM = 2,          /* device or host allocation failed */
  MF_ERR_NONFINITE = 3,    /* a non-finite value appeared in the updated state */
  MF_ERR_NEG_STATE = 4,    /* density or pressure <= 0 after the positivity fix, or dt <= 0 */
  MF_ERR_TIMEOUT = 5,      /* a bounded wait on the device gave up */
  MF_ERR_CUDA = 6,         /* a CUDA runtime call failed */
  MF_ERR_UNSUPPORTED = 7,  /* option combination not implemented */
  MF_ERR_SCRATCH_LIMIT = 8, /* mf_patch_update_noalloc: the patch needs more scratch than
                               MF_NOALLOC_SCRATCH_BYTES */
  MF_ERR_NO_ROOM = 9         /* mf_server_admit: no free run slot or arena space (retry later) */
} mf_status;

/* time_approximation (PatchMHDAM::eTimeApproximation) */
enum { MF_TA_FIRST_ORDER = 0, MF_TA_HANCOCK = 1, MF_TA_RK2 = 2 };
/* Precision modes.
   MF_PREC_FP64       FP64 everywhere, every operation in the reference's order
                      and rounding (no fused multiply-add): the parity path.
   MF_PREC_MIXED      FP32 reconstruction, Riemann fluxes and CFL wave speeds;
                      conserved state, flux-divergence accumulation, pressure
                      recovery, positivity fix and the charge-exchange rates
                      FP64.
   MF_PREC_FP64_FAST  FP64 everywhere with fused multiply-adds and reused
                      reciprocals (results differ from MF_PREC_FP64 at the
                      rounding level; limiter and region decisions identical
                      for identical input states).
   MF_PREC_MIXED_CE32 MF_PREC_MIXED with the charge-exchange rates in FP32 as
                      well (opt-in: the rates are the dominant FP64 work of the
                      update; the source they scale is still added to the
                      FP64 state in FP64). */
enum { MF_PREC_FP64 = 0, MF_PREC_MIXED = 1, MF_PREC_FP64_FAST = 2, MF_PREC_MIXED_CE32 = 3 };
/* physical (non-periodic) boundary treatment of primitive ghost cells */
enum { MF_BC_NONE = 0, MF_BC_FARFIELD = 1 };
/* limiter1D::eLimiters (src/limiter1D.H:17-28) */
enum {
  MF_LIM_CD = 0, MF_LIM_MINMOD = 1, MF_LIM_SUPERBEE = 2, MF_LIM_VANALBADA = 3,
  MF_LIM_MC = 4, MF_LIM_HARMONIC = 5, MF_LIM_HYPERBEE = 6, MF_LIM_KOREN = 7,
  MF_LIM_VENKATAKRISHNAN = 8, MF_LIM_VANLEER = 9, MF_LIM_WENO3 = 10, MF_LIM_WENO3YC = 11
};

#define MF_MAX_FLUIDS 5
/* plasma (8) + psi (1) + 4 neutral fluids x 5 */
#define MF_MAX_COMP 29

typedef struct mf_box {
  int lo[3];
  int hi[3];   /* inclusive, cell-centred */
} mf_box;

typedef struct mf_fab {
  double* data;  /* component-major, x fastest */
  mf_box box;    /* box of the stored data (valid box + ghosts) */
  int ncomp;
} mf_fab;

typedef struct mf_params {
  int space_dim;           /* 2 or 3 */
  int n_fluids;            /* 1 = MHD plasma only; 2..5 = plasma + (n_fluids-1) neutral H fluids */
  int time_approximation;  /* MF_TA_FIRST_ORDER or MF_TA_RK2 */
  int flux;                /* mhdam.flux: 0/1 Roe 8-wave arithmetic avg, 3 Roe 8-wave Roe avg,
                              2/4 Rusanov (arith/Roe avg), 11/13 Roe 7-wave (arith/Roe avg) */
  int divb_cleaning;       /* eDivergenceCleaning (src/PatchMHDAM.H:43-50): 0 none;
                              1-3 constrained transport with the edge field of
                              Balsara-Spicer (1) or Gardiner-Stone (2, 3; 2D only:
                              the reference's 3D routines store the z-edge field
                              through EX); 5 GLM/Dedner (Roe 7-wave + 2x2 (Bn,psi)
                              flux); 4 (projection) is not supported */
  int use_8wave;           /* Powell 8-wave source (mhdam.8wave_use) */
  int divb_method;         /* 0: none; 1: Bn = average of face states; 2: central */
  int limiter[8];          /* limiter per plasma primitive rho,u,v,w,p,bx,by,bz */
  int check_positivity;    /* first-order fallback where rho or p face values <= 0 */
  int precision;           /* MF_PREC_FP64 or MF_PREC_MIXED */
  double gamma;
  double smallr, smallp;   /* EOS floors */
  double entropy_fix;      /* del2 of the Roe solvers (mhdam.entropy_fix_coeff, default 0.3) */
  double small_b;          /* smallB of the Roe solvers (1e-9) */
  double dx;               /* uniform cell size */
  double dedner_ch, dedner_cp;   /* current GLM speeds (SETDEDNERCONST) */
  double factor_ch, factor_cp;   /* Ch = factor_ch*dx/dt, Cp = sqrt(Ch*dx/factor_cp) */
  /* charge exchange between the plasma and each neutral fluid */
  int charge_exchange;
  double ce_scale_vel;     /* velocity scale applied before the cross-section */
  double ce_sigma_scale;   /* cross-section scale (length x number density units) */
  double ce_sigma_a, ce_sigma_b;   /* sigma(v) = scale*(a - b ln(v*scale_vel))^2 * damping */
  double ce_damp_c, ce_damp_pow;   /* damping (1-exp(-c/(v*scale_vel)))^pow when c > 0 */
  /* region classification (DEFINE_REGIONS_2F) */
  double sun_center[3];    /* x = (i+1/2)dx - sun_center[0], ... */
  double sun_r;            /* sunR */
  double sun_v;            /* sunV; LIMSUN = 0.6 sunV */
  double region_t_coeff;   /* TEMP = region_t_coeff * p / rho */
  double region_tmlim;     /* TMLIM */
  double region_zbot, region_ztop;  /* RegSafeZBot / RegSafeZTop (3D) */
  /* inner solar-wind sphere reset after each stage (HELIOREINIT_DEFAULT; field
     polarity: sun_b_monopolar below) */
  int reinit_sphere;
  double reinit_r0;        /* Rinit */
  double sun_int_bc_radius;
  double sun_rho, sun_p, sun_b, sun_beta, dir_br;
  /* problem domain (index space) */
  int domain_lo[3], domain_hi[3];
  int periodic[3];
  int bc_kind;             /* MF_BC_NONE or MF_BC_FARFIELD */
  double bc_plasma[8];     /* far-field plasma primitives rho,u,v,w,p,bx,by,bz */
  double bc_neutral1[5];   /* far-field primitives of neutral fluid 1 */
  /* characteristic reconstruction of the plasma variables (mhdam.char_reconstruction,
     Reconstruction::faceValues, src/Reconstruction.cpp:178-203) and its TVD check
     (mhdam.check_tvd: 1 = the 8 plasma variables, 2 = density and pressure) */
  int char_reconstruction;
  int check_tvd;
  /* heliosphere boundary fluxes (HeliosphericProblem::fluxBC -> HELIOBC,
     swlism/HeliosphericProblem.cpp:1994-2188, swlism/HeliosphericF.ChF:221-910):
     with MF_BC_FARFIELD, the fluxes of the faces on the domain boundary are
     replaced by the heliosphere's characteristic boundary fluxes (plasma:
     BFLUXR at the low-x exit, the exact far-field flux at the high-x inflow,
     BFLUX on the other sides; neutrals: van Leer with outflow copy for fluid 1
     (and 4), one-way outflow for fluids 2 and 3).  0 keeps the Riemann fluxes
     of the ghost-filled states. */
  int helio_bc;
  /* neutral pass-through at the sun (HeliosphericProblem::postTimeStep ->
     NEUTRALS_SUNBC, swlism/HeliosphericProblem.cpp:2472-2535,
     swlism/SWLISMF.ChF:1555-1598; strips :489-527): after every level step,
     the cells of the inner sphere (radius sun_r) downstream of the sun
     (x >= sun) take neutral fluid 1 (and 4 with 5 fluids) from the cell
     mirrored across the sun's x plane, y and z momenta reversed.  Level
     steps only (it is a level post-processing in the reference); the sun
     centre must lie on a grid node. */
  int neutral_sun_bc;
  /* tracking surfaces (level sets; mhdam.num_tracking_surfaces and
     mhdam.region_tracer, main/MHDAM.cpp:709-718): components after the last
     fluid, carried by the plasma velocity (PhysProblem::lsIndexField,
     src/PhysProblem.cpp:327-330).  Face values with limiter_ls, upwind face
     value by the sign of sqrt(rho_L) u_L + sqrt(rho_R) u_R (LEVELSETFLUX,
     src/LevelSetF.ChF:37-105), non-conservative update
     phi -= dt/dx u (F(i+1) - F(i)) with the stage-start cell velocity
     (UPDATELEVELSET :200-234; Hancock: FLUXESHANCOCK_LS :9-35 and
     UPDATELEVELSETHANCOCK :354-388), then the floor of POSTPROCESSING_LS
     (:426-465).  Not refluxed at coarse-fine faces (the flux registers cover
     the fluid components only).  At most 2; plasma, psi, neutrals and
     surfaces together at most MF_MAX_COMP. */
  int num_tracking_surfaces;
  int limiter_ls;          /* mhdam.limiter_LS (the reference reads it into the variable of
                              the other limiter keys, so a deck without it takes the last
                              limiter key read) */
  /* 1: the last tracking surface is the heliosphere's region tracer
     (HeliosphericProblem::defineRegions with m_region_tracer,
     swlism/HeliosphericProblem.cpp:2538-2575 -> DEFINE_REGIONS_TRACER_4F,
     swlism/SWLISMF.ChF:839-1016): negative = solar wind (regions 2/3 by the
     radial speed and temperature, 4 outside the z band), positive =
     interstellar (1, or 4 where the flow is dense, slow, deflected from
     lism_u or hot); far-field ghosts hold +1 (HELIOGS). */
  int region_tracer;
  double lism_u[3];        /* lismUX, lismUY, lismUZ: interstellar flow direction */
  /* Growth cap of the time step that a level chains on the device
     (AMR_MHDAM::assignDt, srcIdeal/AMR_MHDAM.cpp:1614-1624,1680; input key
     max_dt_growth, default 1.1 at :94-95): the next dt of mf_level_step_async
     and of a served run is min(cfl * dt_min, max_dt_growth * dt), and
     mf_hier_assign_dt caps the next coarse dt the same way.  <= 0: no cap. */
  double max_dt_growth;
  /* Polarity of the inner-sphere field of HELIOREINIT_DEFAULT
     (swlism/HeliosphericPlasmaBCF.ChF:1435-1566): 1 monopolar; 0 bipolar, the
     reference default (HeliosphericProblem sets m_sunBmonopolar = -1 and maps
     every value but 1 to 0, swlism/HeliosphericProblem.cpp:106,151,156).
     Bipolar: B keeps its sign where the colatitude theta is below the
     current-sheet colatitude thetaS(r, phi, t) and flips elsewhere, and the
     heliospheric-current-sheet surface iHCS (the first tracking surface;
     with the region tracer, the first of two) is set to +1 / -1 there. */
  int sun_b_monopolar;
  double sun_tilt;         /* sunTILT: tilt of the current sheet, degrees */
} mf_params;

struct mf_ctx;
struct mf_level;
typedef struct mf_ctx mf_ctx;
typedef struct mf_level mf_level;

/* Defaults of the reference driver (main/MHDAM.cpp:647-666, 913-1046):
   flux 1, minmod for all variables, first-order time, divB method 1, 8-wave on,
   entropy fix 0.3, smallB 1e-9, gamma 5/3, periodic unit domain of 64 cells. */
void mf_params_default(mf_params* p, int space_dim, int n_fluids);

/* Number of conserved components for the parameter set (EqSysMHDMF ctor,
   srcIdeal/EqSysMHDMF.cpp:11-48). */
int mf_params_num_cons(const mf_params* p);

mf_status mf_create(const mf_params* p, mf_ctx** out);
void mf_destroy(mf_ctx* ctx);
int mf_num_ghost(const mf_ctx* ctx);
int mf_num_cons(const mf_ctx* ctx);
mf_status mf_set_current_time(mf_ctx* ctx, double t);
mf_status mf_set_dedner(mf_ctx* ctx, double ch, double cp);
const char* mf_status_string(mf_status s);
/* Upper bound (seconds) of every host wait on the device; a wait that runs
   out returns MF_ERR_TIMEOUT and leaves the work queued.  Default 600 s or
   the MF_WAIT_TIMEOUT_S environment variable.  No reference counterpart (the
   reference has no device). */
mf_status mf_set_wait_timeout(mf_ctx* ctx, double seconds);

/* One time step of one patch, in place on U's valid box (same semantics as
   PatchMHDAM::updateState).  U: device fab holding valid + mf_num_ghost()
   ghost layers with the ghosts already filled by the caller.  F: NULL or an
   array of space_dim device fabs sized on the faces of `valid` in each
   direction (node-centred box), receiving the fluxes used for the update
   (RK2: average of both stages).  divB: NULL or a device fab on `valid`.
   new_dt / min_cell: patch minimum of dx / (max wave speed) and its cell
   (first minimum in Fortran order).  stream: cudaStream_t or NULL.
   The call returns after the stream has finished. */
mf_status mf_patch_update(mf_ctx* ctx, mf_fab* U, const mf_box* valid, double dt,
                          mf_fab* F, mf_fab* divB, double* new_dt, int min_cell[3],
                          void* stream);

/* mf_patch_update with updateState's EdgeBox argument (src/PatchMHDAM.H:
   252-260): with constrained transport (divb_cleaning 1-3), E receives the
   edge field of the step (the average of the two RK2 stages' fields, or the
   one stage's), as EdgeBox fabs on `valid`: in 3D three device fabs,
   E[d] on the valid box made nodal in the two directions other than d; in
   2D one nodal fab E[0].  E may be NULL; without constrained transport it is
   not touched. */
mf_status mf_patch_update_e(mf_ctx* ctx, mf_fab* U, const mf_box* valid, double dt,
                            mf_fab* F, mf_fab* divB, mf_fab* E, double* new_dt,
                            int min_cell[3], void* stream);

/* PatchMHDMF::recalculateMagneticField (srcIdeal/PatchMHDMF.cpp:1461-1484 ->
   recalculateB, srcIdeal/DivCleaningF.ChF:4-72): on `box`, B = Uold's B minus
   dt times the discrete curl of the edge field E (EdgeBox fabs as above),
   and U's energy keeps its non-magnetic part.  What AMRLevelIdealMHD::
   postTimeStep does after a level step with constrained transport
   (srcIdeal/AMRLevelIdealMHD.cpp:1649-1688), with the level's UOld.
   Requires divb_cleaning 1-3. */
mf_status mf_recalculate_magnetic_field(mf_ctx* ctx, mf_fab* U, const mf_fab* Uold,
                                        const mf_fab* E, double dt, const mf_box* box,
                                        void* stream);

/* Size of the device scratch array of mf_patch_update_noalloc: 16 MiB, enough
   for a 16^3 patch of the 24-component multi-fluid model with 4 ghost layers
   (about 12.7 MiB) or a 2D single-fluid patch of about 200^2 cells. */
#define MF_NOALLOC_SCRATCH_BYTES (16u << 20)

/* mf_patch_update for callers that cannot allocate device memory: processes
   whose device memory belongs to a pool allocator that must not be bypassed
   (the host application owns all of HBM), and real-time or serving loops that
   forbid allocation after start-up.  No counterpart in the reference (its
   patch update allocates its temporaries on every call).  Same arguments and
   results as mf_patch_update; it calls no cudaMalloc, cudaFree or other
   allocating routine.  Its scratch is one file-scope device array of
   MF_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
   the process exits; a patch that needs more returns MF_ERR_SCRATCH_LIMIT.
   The Hancock time approximation and constrained transport (divb_cleaning
   1-3) return MF_ERR_UNSUPPORTED.  In mixed precision the flux kernels
   convert W to FP32 face by face instead of reading a stored FP32 copy of W
   (the same values; the copy would not fit the array).  The first call on a
   device looks the array's device address up (cudaGetSymbolAddress) and
   should come before any stream capture; the device must not be reset while
   the library is in use.  All calls share the array and it keeps the last
   call's contents; calls that overlap on the GPU race and must be
   serialised by the caller.  The call returns after the stream has finished
   (a bounded wait: MF_ERR_TIMEOUT, as mf_set_wait_timeout sets). */
mf_status mf_patch_update_noalloc(mf_ctx* ctx, mf_fab* U, const mf_box* valid, double dt,
                                  mf_fab* F, mf_fab* divB, double* new_dt, int min_cell[3],
                                  void* stream);

/* dx / max wave speed minimum over `box` (PatchMHDMF::computeDt). */
mf_status mf_compute_dt(mf_ctx* ctx, const mf_fab* U, const mf_box* box, double* dt,
                        int min_cell[3], void* stream);

/* A level: all patches of one refinement level resident on the device, one
   contiguous allocation, patch p at offset mf_level_patch_offset(p) doubles. */
mf_status mf_level_create(mf_ctx* ctx, int npatch, const mf_box* valid, mf_level** out);
void mf_level_destroy(mf_level* lev);
long long mf_level_num_doubles(const mf_level* lev);
long long mf_level_patch_offset(const mf_level* lev, int patch);
mf_status mf_level_patch_fab(const mf_level* lev, int patch, mf_fab* out);
long long mf_level_num_cells(const mf_level* lev);
/* Copy the whole level state host -> device / device -> host (layout as on the device). */
mf_status mf_level_upload(mf_level* lev, const double* host, void* stream);
mf_status mf_level_download(const mf_level* lev, double* host, void* stream);
/* The valid cells only, packed on the host: patch p's valid box at
   mf_level_valid_offset(p) doubles, component-major, x fastest (a LevelData
   without ghosts).  One host copy through a device staging buffer (allocated
   at the first call) and a scatter / gather kernel.  Ghost cells are not
   transferred: the level step fills them by its exchange; those outside a
   non-periodic domain keep what the last full upload placed there (zero on a
   new level). */
long long mf_level_valid_doubles(const mf_level* lev);
long long mf_level_valid_offset(const mf_level* lev, int patch);
mf_status mf_level_upload_valid(mf_level* lev, const double* host, void* stream);
mf_status mf_level_download_valid(mf_level* lev, double* host, void* stream);
/* Fill ghost cells of every patch from the valid cells of its neighbours
   (periodic images included); LevelData::exchange. */
mf_status mf_level_exchange(mf_level* lev, void* stream);
/* Level minimum of dx / max wave speed over the valid cells (the initial dt of
   AMRLevelIdealMHD::computeInitialDt, srcIdeal/AMRLevelIdealMHD.cpp:2140-2200). */
mf_status mf_level_compute_dt(mf_level* lev, double* dt, int* min_patch, int min_cell[3],
                              void* stream);
/* One time step of every patch of the level: exchange, both RK2 stages (or the
   first-order stage), and the level minimum of the new dt.  The step is
   replayed from a CUDA graph after its first call.  new_dt: level minimum of
   dx/cmax (before cfl); min_patch/min_cell: where it was attained. */
mf_status mf_level_step(mf_level* lev, double dt, double* new_dt, int* min_patch,
                        int min_cell[3], void* stream);
/* Enqueue one step without waiting: dt and the GLM speeds are read from the
   device copy written by the previous step (dt = cfl * previous minimum,
   capped at max_dt_growth times the previous dt as AMR_MHDAM::assignDt does;
   Ch = factor_ch*dx/min, Cp = sqrt(Ch*dx/factor_cp)).  Call
   mf_level_seed_dt first, mf_level_result to read the outcome. */
mf_status mf_level_seed_dt(mf_level* lev, double dt, double cfl, void* stream);
mf_status mf_level_step_async(mf_level* lev, void* stream);
mf_status mf_level_result(mf_level* lev, double* new_dt, int* min_patch, int min_cell[3],
                          void* stream);
/* Time of the level's state (AMRLevel::time, passed to the patch update by
   AMRLevelIdealMHD::advance as setCurrentTime, srcIdeal/AMRLevelIdealMHD.cpp:
   854): the start time of its next step.  A new level starts at the
   context's current time (mf_set_current_time); every step advances it by
   its dt (on the device for the async form).  The time enters the bipolar
   inner-sphere field (HELIOREINIT_DEFAULT at time + stage dt).
   mf_level_time waits for the level's queued work. */
mf_status mf_level_set_time(mf_level* lev, double time);
mf_status mf_level_time(mf_level* lev, double* time);
/* Kernel launches enqueued by one mf_level_step (for accounting). */
int mf_level_launches_per_step(const mf_level* lev);
/* Schedule of the level's stages (no reference counterpart; the results do
   not depend on it beyond FP32 rounding of the fluxes).  tile = {0,0,0}: the
   split kernels (face fluxes of each direction in HBM, then the update);
   tile = a shape in cells (x, y, z; z ignored in 2D; at most 256 cells and
   the shared memory of two blocks per SM): one fused kernel per stage that
   computes the fluxes of each tile in shared memory and updates it.  The
   fused kernel covers MF_PREC_MIXED and MF_PREC_MIXED_CE32 with RK2 or first
   order, without constrained transport, characteristic reconstruction,
   tracking surfaces or central Bn (else MF_ERR_UNSUPPORTED); while a
   hierarchy's flux registers are attached the level uses the split kernels.
   Levels start with the split kernels; mf_level_autotune picks the
   schedule by timing.  mf_level_schedule returns the current tile
   ({0,0,0}: split). */
mf_status mf_level_set_schedule(mf_level* lev, const int tile[3]);
mf_status mf_level_schedule(const mf_level* lev, int tile[3]);

/* Face-flux form of the FP64 paths (MF_PREC_FP64 and MF_PREC_FP64_FAST; no
   reference counterpart; results unchanged, bit for bit).  MF_FLUX_FACES: one
   thread per face, which evaluates the limited face values of both cells
   beside it.  MF_FLUX_LINES: a block takes whole lines of faces along the
   direction and computes each cell's limited face values once, in shared
   memory, before the Riemann fluxes.  RK2 and first order (Hancock keeps
   its own face-value arrays); MF_ERR_UNSUPPORTED for mixed precision, for
   Hancock, and for a patch longer than 254 cells along a direction.  Levels
   start with MF_FLUX_FACES; mf_level_autotune picks the form by timing. */
enum { MF_FLUX_FACES = 0, MF_FLUX_LINES = 1 };
mf_status mf_level_set_flux_form(mf_level* lev, int form);
mf_status mf_level_flux_form(const mf_level* lev, int* form);

/* Overlap of the split flux and update kernels (no reference counterpart;
   results unchanged, bit for bit).  chunks = 1: one flux launch per direction
   and one update launch per stage.  chunks = 2..MF_MAX_OVERLAP_CHUNKS: the
   level's patches are cut into about that many chunks of consecutive patches
   (each starting on a multiple of 256 cells; fewer where the patches do not
   allow more) and each stage runs chunks + 1 launches, launch k computing
   the FP32 fluxes of chunk k and the update of chunk k - 1 in one grid of
   alternating blocks, so that the FP64-bound update and the FP32 fluxes
   share the SMs.  MF_PREC_MIXED and MF_PREC_MIXED_CE32 with RK2 or first
   order and without constrained transport (else MF_ERR_UNSUPPORTED); the
   fused schedule and attached flux registers use unchunked launches.  mf_level_overlap returns the current chunk count;
   mf_level_autotune picks it by timing. */
#define MF_MAX_OVERLAP_CHUNKS 8
mf_status mf_level_set_overlap(mf_level* lev, int chunks);
mf_status mf_level_overlap(const mf_level* lev, int* chunks);
/* Diagnostic (no reference counterpart): one step enqueued launch by launch
   (no graph) with a CUDA event after every launch on the launching stream;
   ms[i] is the device time of launch i, kinds[i] its kernel kind (0 ghost
   exchange, 1 primitive variables, 2 face fluxes, 3 update + sources,
   4 dt reduction, 5 hierarchy coupling, 6 problem post-processing,
   7 constrained transport, 8 fused fluxes + update, 9 the fluxes of one
   overlap chunk with the update of the previous one).  The state advances by
   one step with time step dt. */
mf_status mf_level_profile_step(mf_level* lev, double dt, float* ms, int* kinds, int* nlaunch,
                                int max_launch);

/* Riemann fluxes of n face-state pairs in direction dir (device pointers:
   wl, wr = n x nc primitive values laid out face by face, f = n x nc fluxes
   out): the context's plasma solver (RIEMANNF / RIEMANN7F / RUSANOVF), the
   GLM (Bn, psi) flux with the context's Ch (DEDNER2X2F) and the neutral van
   Leer fluxes (VANLEERF), in the context's precision mode; returns after
   the kernel finished.  The per-face form of the fluxes the patch update
   computes, for tests of the solvers in isolation. */
mf_status mf_face_fluxes(mf_ctx* ctx, int dir, int n, const double* wl, const double* wr,
                         double* f, void* stream);

/* Autotuner (no reference counterpart: the reference runs one Fortran call
   per patch).  Times the prim, flux and update kernels of the level's batch
   at 64, 128 and 256 threads per block (reps launches each, stage-1 form, so
   the level's state is not changed) and keeps the fastest shape of each
   kind for later steps.  Where the fused kernel covers the level's options
   (see mf_level_set_schedule) and no flux registers are attached, it then
   times stage 1 with the split kernels against the fused kernel at the tile
   shapes 8x8x4, 8x4x4, 16x8x2, 8x8x2 and 4x4x4 (16x16, 32x8, 16x8, 8x8 in
   2D) that fit, and keeps the fastest schedule (mf_level_schedule reads
   it).  Previously captured step graphs are rebuilt.  threads (nullable)
   receives the chosen {prim, flux, update} shapes.  Results of a step do not
   depend on the shapes; the schedule changes them at most by FP32 rounding
   of the charge-exchange rates in MF_PREC_MIXED_CE32. */
mf_status mf_level_autotune(mf_level* lev, int reps, int threads[3]);

/* ---- Hierarchy: levels coupled across refinement (Berger-Oliger) ----
   levels[0] is the coarsest; level l+1 is refined by ratios[l] with respect
   to level l (its mf_params: dx = dx_l / ratio, domain refined by ratio, same
   time approximation and precision), each level with its own context.  Fine
   boxes must be aligned to the ratio and properly nested: every coarse cell
   the interpolation stencil, the flux register or the averaging reads must be
   a valid cell of the coarser level (else MF_ERR_BAD_ARG at creation).
   While a hierarchy exists its levels copy the fluxes of the register faces
   out of every step (extra gather launches); destroy it before the levels. */
typedef struct mf_hier mf_hier;
mf_status mf_hier_create(int nlevels, mf_level* const* levels, const int* ratios,
                         mf_hier** out);
void mf_hier_destroy(mf_hier* h);
/* Level times (all levels start at the same time; default 0). */
mf_status mf_hier_set_time(mf_hier* h, double time);
mf_status mf_hier_times(const mf_hier* h, double* times);
/* One step dt0 of level 0 (AMR_MHDAM::timeStep): level l advances
   ratio[l-1] times per step of level l-1 with dt_l = dt_{l-1} / ratio.
   Before each level step its ghost cells over coarse cells not covered by the
   finer level are interpolated from the coarser level (in time between its
   states before and after its step, in space with limited slopes and, with
   GLM, the divergence correction of the B slopes); after the finer level has
   caught up, the coarse cells next to the fine region are refluxed with the
   fine fluxes and the covered coarse cells are averaged from the fine cells.
   With GLM (divb_cleaning 5) and factor_ch > 0, Ch and Cp of every level are
   set from level 0's new dt after its step, as the reference does.
   new_dt: min over levels of the level's dx/cmax times its refinement with
   respect to level 0 (multiply by the CFL number for the next dt0).
   Synchronous: returns after the step finished. */
mf_status mf_hier_step(mf_hier* h, double dt0, double* new_dt, void* stream);
/* The next coarse time step after mf_hier_step (AMR_MHDAM::assignDt with
   subcycling, srcIdeal/AMR_MHDAM.cpp:1570-1660): cfl times the new_dt of the
   last step, capped at max_dt_growth (level 0's parameters) times the last
   step's dt0.  MF_ERR_BAD_ARG before the first step. */
mf_status mf_hier_assign_dt(const mf_hier* h, double cfl, double* dt0);
/* The coupling operations on their own: copy the coarse values that the
   interpolation onto level+1 reads (the "old" coarse state); interpolate the
   coarse-fine ghosts of level (>= 1) with time fraction alpha between that
   copy and the current coarse state; average level+1 onto level. */
mf_status mf_hier_snapshot(mf_hier* h, int level, void* stream);
mf_status mf_hier_fill_ghosts(mf_hier* h, int level, double alpha, void* stream);
mf_status mf_hier_average_down(mf_hier* h, int level, void* stream);
/* Sizes of the coupling of levels (pair, pair+1): interpolation sites,
   interpolated fine cells, register faces, refluxed cells, averaged cells,
   coarse cells read by the interpolation. */
mf_status mf_hier_info(const mf_hier* h, int pair, long long counts[6]);
int mf_hier_launches_per_step(const mf_hier* h);

/* ---- Serving: independent runs stepped together in shared launches ----
   No reference counterpart (the reference advances one simulation per
   process).  A server keeps every admitted run resident in device arenas
   sized once from an HBM budget and advances all of them with one set of
   batched launches per step: a run is a level of patches covering its own
   domain [0, n-1]^d, with the physics of the server's context (equations,
   solvers, limiters, sources, inner sphere) and its own grid size, spacing,
   far-field state, CFL number, dt and GLM speeds.  The numbers of a run do
   not depend on which other runs share its launches.  Calls on one server
   are not thread-safe. */
typedef struct mf_server mf_server;

typedef struct {
  int n[3];              /* cells per direction; 1 for unused directions */
  int patch;             /* patch edge length (the last patch of a row may be shorter) */
  double dx;             /* grid spacing */
  double cfl;            /* dt of each step = cfl * dx / (largest signal speed) */
  double bc_plasma[8];   /* far-field primitive states (MF_BC_FARFIELD contexts) */
  double bc_neutral1[5];
} mf_run_spec;

mf_status mf_server_create(mf_ctx* physics, double hbm_budget_bytes, int max_runs,
                           mf_server** out);
void mf_server_destroy(mf_server* srv);
/* Device bytes a run of this spec holds while admitted (-1: invalid spec). */
long long mf_server_run_bytes(const mf_server* srv, const mf_run_spec* spec);
/* Largest free cell range of the arena, in bytes of the cell arrays (U, U1, W,
   and the FP32 copy of W in mixed precision). */
long long mf_server_free_bytes(const mf_server* srv);
/* Admit a run whose initial conserved state is `state` (host: the run's
   domain as one FArrayBox without ghosts, nc components, x fastest).  Waits
   for the server's queued work.  MF_ERR_NO_ROOM: no slot or arena space. */
mf_status mf_server_admit(mf_server* srv, const mf_run_spec* spec, const double* state,
                          int* run);
/* Enqueue one step of every admitted run on the stream (asynchronous). */
mf_status mf_server_step(mf_server* srv, void* stream);
/* Wait for the enqueued steps and fetch every run's last results. */
mf_status mf_server_sync(mf_server* srv, void* stream);
/* Steps taken, dt_min of the last synced step, and the run's status. */
mf_status mf_server_run_info(const mf_server* srv, int run, long long* steps, double* dt_min,
                             mf_status* run_status);
/* Copy the run's state to `state` (nullable; layout of mf_server_admit) and
   release its slot and arena ranges. */
mf_status mf_server_retire(mf_server* srv, int run, double* state, void* stream);
int mf_server_active(const mf_server* srv);
/* CUDA stream priority of the server's launches (lower = more urgent,
   clamped to the device's range): servers of short runs given a higher
   priority than servers of long runs finish their runs first when both
   share the GPU. */
mf_status mf_server_set_priority(mf_server* srv, int priority);

/* Problem set-up on host fabs (PhysProblem::initialize):
   Orszag-Tang vortex (problems/OrszagF.ChF:27-79) and the synthetic
   heliosphere (uniform inflow + inner solar-wind sphere). */
mf_status mf_init_orszag_host(const mf_params* p, mf_fab* U, const mf_box* box);
mf_status mf_init_helio_host(const mf_params* p, const double* inflow_plasma,
                             const double* inflow_neutrals, mf_fab* U, const mf_box* box);

#ifdef __cplusplus
}
#endif
#endif
