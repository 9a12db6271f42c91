/*
 * g3m3.h -- C ABI of the GB300-native G3M^3 multifluid step
 * (libg3m3_gpu.so, sm_103a).
 *
 * Two layers:
 *
 * 1. Drop-in routines.  One entry point per reference subroutine on the
 *    time-step path, taking the reference's dummy arguments in the same
 *    order (file:line of each below).  Arrays follow the Fortran layout
 *    A(nx,ny,nz,n_grids) / A(nx,ny,nz), column-major FP32, and may be either
 *    device pointers or host arrays.  A host array is mirrored on the device
 *    the first time the library sees it (keyed by its base address) and
 *    stays resident; results are written to the mirror.  Call
 *    g3m3_sync_to_host() before host code reads an array the library wrote,
 *    and g3m3_sync_to_device() after host code changed an array the library
 *    has mirrored.  Scalars the Fortran only reads are passed by value;
 *    scalars it returns are pointers.  Every routine returns a status
 *    (G3M3_OK = 0); g3m3_last_error() describes the last failure.  The
 *    reference prints and stops instead (3d_main.f90:1970-1974); a caller
 *    keeps that behaviour by stopping on a nonzero status.
 *
 * 2. The step engine.  g3m3_model_* keeps a whole multi-box state on the
 *    device and runs the reference's main loop (3d_main.f90:1925-3095: time
 *    step schedule, sub-cycling, predictor, corrector, Lapidus smoothing,
 *    flux correction, boundaries, nested-grid sync) with fused kernels,
 *    buffer rotation instead of store_array copies, and optionally one CUDA
 *    graph per main step.
 *
 * Threading: a context has one CUDA stream and must not be used from two
 * host threads at once.  All calls are asynchronous on that stream unless
 * they return a host value.
 */
#ifndef G3M3_H
#define G3M3_H

#include <stddef.h>
#include <stdint.h>

#include "g3m3_types.h"

#ifdef __cplusplus
extern "C" {
#endif

#define G3M3_OK 0
#define G3M3_ERR_ARG 1       /* bad dimensions, box index or pointer      */
#define G3M3_ERR_CUDA 2      /* a CUDA call failed                        */
#define G3M3_ERR_NOCONV 3    /* div B solver stopped without converging   */
#define G3M3_ERR_NONFINITE 4 /* a check found NaN or Inf                  */
#define G3M3_ERR_ALLOC 5     /* device allocation failed                  */
#define G3M3_ERR_STATE 6     /* call out of order                         */

typedef struct g3m3_ctx g3m3_ctx;
typedef struct g3m3_model g3m3_model;
typedef struct g3m3_ensemble g3m3_ensemble;

/* ---- context -------------------------------------------------------- */
int g3m3_ctx_create(g3m3_ctx** out, int device);
int g3m3_ctx_destroy(g3m3_ctx* ctx);
const char* g3m3_last_error(g3m3_ctx* ctx);
/* Copy the device mirror of a host array back to it / refresh the mirror
 * from the host array.  Device pointers are accepted and ignored. */
int g3m3_sync_to_host(g3m3_ctx* ctx, void* host_array);
int g3m3_sync_to_device(g3m3_ctx* ctx, const void* host_array);
/* Drop every mirror (their device memory is freed). */
int g3m3_release_mirrors(g3m3_ctx* ctx);
int g3m3_synchronize(g3m3_ctx* ctx);
/* Library build description (kernel arch, flags). */
const char* g3m3_version(void);
/* The context's CUDA stream (cudaStream_t), for event timing by callers. */
void* g3m3_ctx_stream(g3m3_ctx* ctx);

/* Failure handling.  The reference stops or warns where these report a
 * status (3d_main.f90:1970-1974; sub_sparse_solver.f90:93,157).
 * - g3m3_ctx_set_cg_maxit: cap every div B / sparse_solver solve of the
 *   context at `maxit` iterations (0 restores the reference's 10*npts,
 *   sub_sparse_solver.f90:80); a solve that reaches the cap returns
 *   G3M3_ERR_NOCONV, the reference's "too many iterations" warning.
 * - g3m3_ctx_set_finite_check: when on, FP32 arrays staged from the host
 *   (first mirror upload, g3m3_sync_to_device, g3m3_model_set_field/state,
 *   g3m3_model_step_host) are scanned and a NaN or Inf returns
 *   G3M3_ERR_NONFINITE before anything is uploaded.  Off by default.
 * - g3m3_ctx_set_alloc_limit: a budget in bytes for the device memory the
 *   context (and its models) may allocate (0: none); an allocation past it
 *   fails with G3M3_ERR_ALLOC as a full device would.  For testing the
 *   out-of-memory paths. g3m3_ctx_allocated gives the bytes charged so far. */
int g3m3_ctx_set_cg_maxit(g3m3_ctx* ctx, int maxit);
int g3m3_ctx_set_finite_check(g3m3_ctx* ctx, int on);
int g3m3_ctx_set_alloc_limit(g3m3_ctx* ctx, size_t bytes);
size_t g3m3_ctx_allocated(g3m3_ctx* ctx);

/* ---- a1: push_ion -- sub_push_ion.f90:4-17 ---------------------------- */
int g3m3_push_ion(g3m3_ctx* ctx,
    float* qrho, float* qpresx, float* qpresy, float* qpresz,
    float* qpx, float* qpy, float* qpz,
    const float* oldqrho, const float* oldqpresx, const float* oldqpresy,
    const float* oldqpresz, const float* oldqpx, const float* oldqpy,
    const float* oldqpz,
    const float* wrkqrho, const float* wrkqpresx, const float* wrkqpresy,
    const float* wrkqpresz, const float* wrkqpx, const float* wrkqpy,
    const float* wrkqpz,
    float* qpresxy, float* qpresxz, float* qpresyz,
    const float* oldqpresxy, const float* oldqpresxz, const float* oldqpresyz,
    const float* wrkqpresxy, const float* wrkqpresxz, const float* wrkqpresyz,
    const float* bsx, const float* bsy, const float* bsz, const float* btot,
    const float* efldx, const float* efldy, const float* efldz, float rmassq,
    float* qvx, float* qvy, float* qvz,
    const float* tvx, const float* tvy, const float* tvz,
    float gamma, float gamma1,
    int nx, int ny, int nz, int n_grids, int box, float delt, float grav,
    float re_equiv, float reynolds,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax,
    int isotropic);

/* ---- a2: push_elec -- sub_push_elec.f90:4-5 (reads arg 1, writes arg 3) */
int g3m3_push_elec(g3m3_ctx* ctx, const float* wrkepres,
    const float* oldepres, float* epres, const float* evx, const float* evy,
    const float* evz, float gamma, float gamma1, int nx, int ny, int nz,
    int n_grids, int box, float delt, float rx, float ry, float rz);

/* ---- a3: push_bfld -- sub_push_bfld.f90:4-6 --------------------------- */
int g3m3_push_bfld(g3m3_ctx* ctx, float* bx, float* by, float* bz,
    const float* oldbx, const float* oldby, const float* oldbz,
    const float* efldx, const float* efldy, const float* efldz,
    int nx, int ny, int nz, int n_grids, int box, float delt,
    float rx, float ry, float rz);

/* ---- a4: calcur -- sub_calcur.f90:5-6 --------------------------------- */
int g3m3_calcur(g3m3_ctx* ctx, const float* bx, const float* by,
    const float* bz, int nx, int ny, int nz, int n_grids, int box,
    float* curx, float* cury, float* curz, float rx, float ry, float rz);

/* bs = b0 + b, btot = max(|bs|, smallbit) of one box (3d_main.f90:2248-2254;
 * an array statement of the main program, not a subroutine). */
int g3m3_total_b(g3m3_ctx* ctx, const float* bx, const float* by,
    const float* bz, const float* bx0, const float* by0, const float* bz0,
    int nx, int ny, int nz, int n_grids, int box, float smallbit,
    float* bsx, float* bsy, float* bsz, float* btot);

/* ---- a5: fnd_evel -- sub_fnd_evel.f90:4-7; fnd_vtot -- sub_fnd_vtot.f90:4-6 */
int g3m3_fnd_evel(g3m3_ctx* ctx, const float* qpx, const float* qpy,
    const float* qpz, const float* qrho, const float* hpx, const float* hpy,
    const float* hpz, const float* hrho, const float* opx, const float* opy,
    const float* opz, const float* orho, const float* curx,
    const float* cury, const float* curz, float* evx, float* evy,
    float* evz, float* tvx, float* tvy, float* tvz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float reynolds);

int g3m3_fnd_vtot(g3m3_ctx* ctx, const float* qpx, const float* qpy,
    const float* qpz, const float* qrho, const float* hpx, const float* hpy,
    const float* hpz, const float* hrho, const float* opx, const float* opy,
    const float* opz, const float* orho, float* vx, float* vy, float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso);

/* ---- a6: BandE -- sub_BandE.f90:5-10 --------------------------------- */
int g3m3_bande(g3m3_ctx* ctx, float* efldx, float* efldy, float* efldz,
    const float* bsx, const float* bsy, const float* bsz,
    const float* curx, const float* cury, const float* curz,
    const float* evx, const float* evy, const float* evz, const float* btot,
    const float* epres, const float* qrho, const float* hrho,
    const float* orho, const float* rst, float resist, float reynolds,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso,
    const int* ijmid, const int* nummid, const int* ijzero, int mbndry,
    const int* numzero, int mmid, int mzero, float rx, float ry, float rz);

/* ---- a7: fnd_pres -- sub_fnd_pres.f90:5-6 ---------------------------- */
int g3m3_fnd_pres(g3m3_ctx* ctx, const float* px, const float* py,
    const float* pz, const float* pxy, const float* pxz, const float* pyz,
    float* p_para, float* p_perp, float* p_cross,
    const float* vvx, const float* vvy, const float* vvz,
    const float* bxt, const float* byt, const float* bzt,
    int nx, int ny, int nz, int n_grids, int box);

/* ---- a8: lap_plasma -- sub_lap_plasma.f90:4-10; lap_elec :151-152;
 *          lap_bfld :202-203 ---------------------------------------------- */
int g3m3_lap_plasma(g3m3_ctx* ctx, const float* rho, const float* px,
    const float* py, const float* pz, const float* presx,
    const float* presy, const float* presz, const float* presxy,
    const float* presxz, const float* presyz,
    float* wrkrho, float* wrkpx, float* wrkpy, float* wrkpz,
    float* wrkpresx, float* wrkpresy, float* wrkpresz,
    float* wrkpresxy, float* wrkpresxz, float* wrkpresyz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt, int isotropic);

int g3m3_lap_elec(g3m3_ctx* ctx, const float* ppres, float* wrkppres,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt);

int g3m3_lap_bfld(g3m3_ctx* ctx, const float* bx, const float* by,
    const float* bz, float* wrkbx, float* wrkby, float* wrkbz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt);

/* ---- a9: fcsmooth -- sub_fcsmooth.f90:7-8 (tempx..z are scratch) ------
 *          flux_correct -- sub_flux_correct.f90:4-35, the 34 fields as
 *          pointer tables in the field order of g3m3_types.h ------------- */
int g3m3_fcsmooth(g3m3_ctx* ctx, float* px, const float* oldpx,
    const float* wrkpx, int nx, int ny, int nz, int n_grids, int box,
    float chipx, float* tempx, float* tempy, float* tempz);

int g3m3_flux_correct(g3m3_ctx* ctx, float* const cur[G3M3_NFIELDS],
    const float* const wrk[G3M3_NFIELDS], const float* const old[G3M3_NFIELDS],
    int nx, int ny, int nz, int n_grids, int box, float difrho, float diferg);

/* ---- a10: set_rho -- sub_set_rho.f90:5-11 ---------------------------- */
int g3m3_set_rho(g3m3_ctx* ctx, float* qrho, float* qpresx, float* qpresy,
    float* qpresz, float* qpresxy, float* qpresxz, float* qpresyz,
    float rmassq, float* hrho, float* hpresx, float* hpresy, float* hpresz,
    float* hpresxy, float* hpresxz, float* hpresyz, float rmassh,
    float* orho, float* opresx, float* opresy, float* opresz,
    float* opresxy, float* opresxz, float* opresyz, float rmasso,
    float* epres, int nx, int ny, int nz, int n_grids, int box,
    float o_conc);

/* ---- a11: set_speed_agrd -- sub_set_speed_agrd.f90:6-22 --------------
 * The six returned scalars are host pointers (the call synchronizes). */
int g3m3_set_speed_agrd(g3m3_ctx* ctx, int nx, int ny, int nz,
    int n_grids, int box, float rmassq, float rmassh, float rmasso,
    int isotropic, float smallbit, float aniso_limit, float vlim,
    float qvlim, float hvlim, float ovlim, float qclim, float hclim,
    float oclim, float cslim,
    const float* bx, const float* by, const float* bz,
    const float* bx0, const float* by0, const float* bz0,
    float* qrho, float* qpx, float* qpy, float* qpz,
    float* qpresx, float* qpresy, float* qpresz,
    float* qpresxy, float* qpresxz, float* qpresyz,
    float* hrho, float* hpx, float* hpy, float* hpz,
    float* hpresx, float* hpresy, float* hpresz,
    float* hpresxy, float* hpresxz, float* hpresyz,
    float* orho, float* opx, float* opy, float* opz,
    float* opresx, float* opresy, float* opresz,
    float* opresxy, float* opresxz, float* opresyz,
    float* epres, float* btot,
    float* pxmax, float* pymax, float* pzmax, float* csmax, float* alfmax,
    float* fastest);

/* ---- a12: store_array -- sub_store_array.f90:1 (writes argument 1) ---- */
int g3m3_store_array(g3m3_ctx* ctx, float* bx, const float* bx0,
    int nx, int ny, int nz, int n_grids, int box);

/* ---- a13: bndry_outer -- sub_bndry_outer.f90:5-16 (34 fields as a table)
 * ---- a14: bndry_inner -- sub_bndry_inner.f90:5-20 -------------------- */
int g3m3_bndry_outer(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS],
    const float* bx0, const float* by0, const float* bz0,
    const g3m3_params* p);

int g3m3_bndry_inner(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS],
    const float* parm_srf, const float* parm_mid, const float* parm_zero,
    const int* ijsrf, const int* numsrf, const int* ijmid,
    const int* nummid, const int* ijzero, const int* numzero,
    int msrf, int mmid, int mzero, const g3m3_params* p);

/* ---- a15: flanks -- sub_flanks.f90:5-7; bndry_flanks (34 fields) -------
 * t_new/t_old are the reference's real(dp) time arrays (host). */
int g3m3_flanks(g3m3_ctx* ctx, float* wrkrho, const float* rho,
    const float* oldrho, int nx, int ny, int nz, int n_grids, int box,
    const double* t_new, const double* t_old, double t, float* work,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax);

int g3m3_bndry_flanks(g3m3_ctx* ctx, float* const target[G3M3_NFIELDS],
    const float* const cur[G3M3_NFIELDS], const float* const old[G3M3_NFIELDS],
    int nx, int ny, int nz, int n_grids, int box,
    const double* t_old, const double* t_new, double t,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax);

/* ---- a16: corer -- sub_corer.f90:5-6; bndry_corer (34 fields) --------- */
int g3m3_corer(g3m3_ctx* ctx, float* rho, int nx, int ny, int nz,
    int n_grids, int box, const float* grd_xmin, const float* grd_xmax,
    const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
    const float* grd_zmax);

int g3m3_bndry_corer(g3m3_ctx* ctx, float* const f[G3M3_NFIELDS],
    int nx, int ny, int nz, int n_grids, int box,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax);

/* ---- a17: flanks_synced -- sub_flanks_synced.f90:5-6 ----------------- */
int g3m3_flanks_synced(g3m3_ctx* ctx, float* rho, int nx, int ny, int nz,
    int n_grids, int box, const float* grd_xmin, const float* grd_xmax,
    const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
    const float* grd_zmax);

/* ---- a18: divB_correct -- sub_divB_correct.f90:25-27 (with its
 * sparse_solver, sub_sparse_solver.f90:19-20).  The initial iterate is 0
 * (the reference starts from uninitialised memory).  *iters (may be NULL)
 * receives the CG iteration count; G3M3_ERR_NOCONV is returned (with the
 * partially cleaned field written) when the solver stops without meeting
 * its tolerance, which the reference only reports as a warning. */
int g3m3_divb_correct(g3m3_ctx* ctx, int nx, int ny, int nz, int n_grids,
    int box, int nbands, const int* divb_band_pos, const float* xspac,
    float divb_errlim, float* bx, float* by, float* bz, int* iters);

/* ---- flux_counter -- sub_flux_counter.f90:5-8 -------------------------
 * Ion momentum through the walls one cell inside the faces of box `box`,
 * as inflow / outflow per species, scaled by grid_spacing / mass.  Each
 * wall is summed in the reference's serial order, so the six results are
 * the reference's bits; only they are copied back to the host. */
int g3m3_flux_counter(g3m3_ctx* ctx, const float* qpx, const float* qpy,
    const float* qpz, const float* hpx, const float* hpy, const float* hpz,
    const float* opx, const float* opy, const float* opz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float grid_spacing,
    float* qflux_in, float* qflux_out, float* hflux_in, float* hflux_out,
    float* oflux_in, float* oflux_out);

/* ---- a18: sparse_solver -- sub_sparse_solver.f90:19-20 ---------------
 * CGNR on the banded system held in banded_matrix(nbands, npts) (column-
 * major FP32, product as banded_tpose, sub_banded_tpose.f90:6-33:
 * out(i) = sum_b banded_matrix(b, i+pos(b)) x(i+pos(b)), the matrix assumed
 * symmetric as in the reference).  soln_vec is the starting iterate and
 * receives the solution; residual2 receives |A x - divB|^2 of the last
 * iterate.  recurse / redo_lim set the starting restart count as the
 * reference's recursive call does (at most 3 restarts in all).  nbands <= 16.
 * Dot products accumulate in FP64.  G3M3_ERR_NOCONV after 10*npts
 * iterations (the reference only warns). */
int g3m3_sparse_solver(g3m3_ctx* ctx, int nbands, int npts,
    const int* divb_band_pos, float divb_errlim, int recurse, int redo_lim,
    const float* divb, float* soln_vec, float* residual2,
    const float* banded_matrix);

/* ---- fluid files and state comparison -------------------------------
 * The reference's fluid file: Fortran unformatted sequential records (a
 * 4-byte little-endian byte count before and after each): t (real(dp));
 * qrho qpx qpy qpz qpresx qpresy qpresz qpresxy qpresxz qpresyz, the same
 * for h and o; bx by bz epres; bx0 by0 bz0 (each (nx,ny,nz,n_grids) FP32);
 * then one record of parm_srf parm_mid parm_zero ijzero numzero ijmid
 * nummid ijsrf numsrf (3d_main.f90:3305-3349, compare_fluids.f90).  Host
 * arrays; state holds the 34 fields in g3m3_types.h order, b0 three fields.
 * The table record is skipped on reading when parm_srf is NULL.  ctx may be
 * NULL (no error text then); these two calls do not use the GPU. */
int g3m3_fluid_write(g3m3_ctx* ctx, const char* path, const g3m3_params* p,
    double t, const float* state, const float* b0, const float* parm_srf,
    const float* parm_mid, const float* parm_zero, const int* ijzero,
    const int* numzero, const int* ijmid, const int* nummid, const int* ijsrf,
    const int* numsrf, int msrf, int mmid, int mzero);
int g3m3_fluid_read(g3m3_ctx* ctx, const char* path, const g3m3_params* p,
    double* t, float* state, float* b0, float* parm_srf, float* parm_mid,
    float* parm_zero, int* ijzero, int* numzero, int* ijmid, int* nummid,
    int* ijsrf, int* numsrf, int msrf, int mmid, int mzero);
/* Field-by-field comparison of two states on the GPU (compare_fluids.f90's
 * use): for each of nfields arrays a[f], b[f] of (nx,ny,nz,n_grids) and each
 * box, stats[(f*n_grids + box-1)*4 + 0..3] = max |a-b|, sum (a-b)^2,
 * sum a^2 (FP64), number of cells whose values differ (+0 = -0, NaN = NaN). */
int g3m3_diff_fields(g3m3_ctx* ctx, int nfields, const float* const* a,
    const float* const* b, int nx, int ny, int nz, int n_grids, double* stats);

/* ---- g3m3_divb_correct without device allocation (no counterpart in the
 * reference) ------------------------------------------------------------
 * Same arguments, arithmetic and results as g3m3_divb_correct, for callers
 * that must not allocate device memory once they run: a host code that
 * gives the whole device to its own memory pool at start-up, or one that
 * keeps other streams busy and cannot take the device-wide synchronisation
 * cudaMalloc and cudaFree may bring.  g3m3_divb_correct grows scratch with
 * cudaMalloc and copies host arrays into new device buffers; this call does
 * neither.  The solver's state and vectors live in one fixed array inside
 * the library (28 MiB per device), which holds boxes of up to
 * G3M3_NOALLOC_DIVB_MAX_CELLS cells; larger boxes are rejected with
 * G3M3_ERR_ARG.  bx, by, bz must be device (or managed) memory, else
 * G3M3_ERR_ARG; xspac and divb_band_pos may be host or device arrays.
 * Every call looks up the array's address on the context's device.  The
 * first call on a device may load the library's device code that holds
 * the array (CUDA loads modules lazily), and the array's memory is taken
 * then: make that first call at start-up, before the caller's pool claims
 * the device and before any stream capture.  Every call on a device shares
 * the one array, which
 * keeps the last call's contents (each call resets what the solver needs
 * zeroed); calls that overlap in time, from two threads or on two streams,
 * race on it and must be serialised by the caller. */
#define G3M3_NOALLOC_DIVB_MAX_CELLS 1048576
int g3m3_divb_correct_noalloc(g3m3_ctx* ctx, int nx, int ny, int nz,
    int n_grids, int box, int nbands, const int* divb_band_pos,
    const float* xspac, float divb_errlim, float* bx, float* by, float* bz,
    int* iters);

/* ---- the adjoint of the main steps (no counterpart in the reference) ----
 * Gradients of a virtual-spacecraft misfit
 *   L = sum over samples of sum_q (value_q(x_s) - target_q,s)^2,
 *   q = bx, by, bz (the perturbation field) and the total density
 *   qrho + hrho + orho, trilinear in the smallest box holding x_s
 *   (findgrid cft_findgrid.f90:70-126, trilin_interp cft_trilin_interp.f90:
 *   34-54), each sample taken at the end of its main step,
 * with respect to the eight upstream parameters of bndry_outer's wind face
 * (sub_bndry_outer.f90:50-103: srho, spx, spy, spz, spress, sbx_wind,
 * sby_wind, sbz_wind) and to the model's state before the first step.
 * g3m3_adjoint_forward runs nsteps main steps from the model's state
 * (host-launched; the schedule of time steps recorded, or the one given;
 * the state kept every checkpoint_every steps) and returns L.
 * g3m3_adjoint_backward restores each checkpoint, re-runs its steps under
 * the recorded schedule with the snapshots the reverse needs, and runs the
 * hand-written reverse of every kernel backwards; it returns dL/dparams
 * (8 doubles), dL/dstate ((34, n_grids, nz, ny, nx) floats, host or
 * device) and dL/d(wrk epres) (the one wrk field the first step reads),
 * and leaves the model at the end of the run.  The time steps are held
 * fixed; the div B solves are reversed as exact linear solves with the
 * forward's CG at cg_errlim (0: the model's divb_errlim); a reversed solve
 * that hits the iteration cap makes backward return G3M3_ERR_NOCONV after
 * finishing.  Requires mbndry = 1 and inner-boundary lists of distinct
 * cells.  Device memory: the checkpoints, and for the steps of one
 * checkpoint interval 8 snapshots of 34 fields per box-step
 * (g3m3_adjoint_tape_bytes). */
typedef struct g3m3_adjoint g3m3_adjoint;
int g3m3_adjoint_create(g3m3_model* m, int nsteps, int checkpoint_every,
    float cg_errlim, g3m3_adjoint** out);
int g3m3_adjoint_destroy(g3m3_adjoint* a);
/* n samples: xyz(3,n) in planet radii, step(n) in 1..nsteps non-decreasing,
 * target(4,n) = bx, by, bz, rho */
int g3m3_adjoint_set_samples(g3m3_adjoint* a, int n, const float* xyz,
    const int* step, const float* target);
int g3m3_adjoint_forward(g3m3_adjoint* a, const double* schedule, double* loss);
/* the recorded schedule: t_stepnew of every box before each main step,
 * (nsteps, n_grids) doubles, for g3m3_adjoint_forward of another run */
int g3m3_adjoint_schedule(g3m3_adjoint* a, double* out);
int g3m3_adjoint_backward(g3m3_adjoint* a, double* grad_params,
    float* grad_state, float* grad_wrk_epres);
size_t g3m3_adjoint_tape_bytes(g3m3_adjoint* a);
/* Wall-clock seconds of the last backward's phases: [0] the re-run of the
 * steps with snapshots, [1] the reverse kernels, [2] the reversed div B
 * passes (their adjoint solves); [3..5] the host time spent issuing each
 * phase's work, before the stream drained (seconds has 6 entries). */
int g3m3_adjoint_phases(g3m3_adjoint* a, double* seconds);
/* Per-stage GPU time of the box-step reverses (CUDA events between the
 * stages; on = 1 turns it on for the next backward, which then waits for
 * each box-step): stage_ms (16, may be null) receives the sums since the
 * last call -- set-up, flux-correction guards, boundaries, fcsmooth,
 * Lapidus guards, boundaries, Lapidus, corrector guards, boundaries,
 * pushes, fields, predictor guards, boundaries, pushes, fields, hand-back. */
int g3m3_adjoint_profile(g3m3_adjoint* a, int on, double* stage_ms);

/* ---- a19: virtual spacecraft -- findgrid cft_findgrid.f90:4 and
 * trilin_interp cft_trilin_interp.f90:10, batched over n trajectory points:
 * xyz(3,n) in planet radii; out(n) = trilinear value of field at each point
 * in the smallest box that contains it (the perturbation field, as
 * cft_craft_handling.f90:178-189 samples it). */
int g3m3_sample_points(g3m3_ctx* ctx, const float* field, int nx, int ny,
    int nz, int n_grids, const float* grid_minvals, const float* grid_maxvals,
    const float* xspac, float re_equiv, const float* xyz, int n, float* out);

/* ---- a20: the step engine -------------------------------------------- */
/* Create a model holding n_grids boxes of the given params on the device.
 * Upload the state with g3m3_model_set_field (cur fields), the dipole with
 * g3m3_model_set_b0 and the inner-boundary lists with
 * g3m3_model_set_inner; then g3m3_model_init_steps. */
int g3m3_model_create(g3m3_ctx* ctx, const g3m3_params* p, g3m3_model** out);
int g3m3_model_destroy(g3m3_model* m);
/* field: 0..33 (g3m3_types.h order); data: A(nx,ny,nz,n_grids), host or
 * device.  which: 0 = current state, 1 = old, 2 = wrk copy. */
int g3m3_model_set_field(g3m3_model* m, int which, int field, const float* data);
int g3m3_model_get_field(g3m3_model* m, int which, int field, float* data);
/* All 34 current fields at once from/to a host block of 34 contiguous
 * A(nx,ny,nz,n_grids) arrays (one copy per direction). */
int g3m3_model_set_state(g3m3_model* m, const float* data);
int g3m3_model_get_state(g3m3_model* m, float* data);
int g3m3_model_set_b0(g3m3_model* m, const float* bx0, const float* by0, const float* bz0);
/* The upstream parameters of bndry_outer's wind face (sub_bndry_outer.f90:
 * 50-103), 8 floats: srho, spx, spy, spz, spress, sbx_wind, sby_wind,
 * sbz_wind; the next main step uses them. */
int g3m3_model_set_wind(g3m3_model* m, const float* wind);
int g3m3_model_set_inner(g3m3_model* m, const float* resistive,
    const int* ijsrf, const int* numsrf, const float* parm_srf, int msrf,
    const int* ijmid, const int* nummid, const float* parm_mid, int mmid,
    const int* ijzero, const int* numzero, const float* parm_zero, int mzero);
/* Guards and first time steps, 3d_main.f90:1861-1903. */
int g3m3_model_init_steps(g3m3_model* m);
/* Run nsteps main steps.  use_graph: 0 = launch kernels from the host loop
 * (plain), 1 = replay one captured CUDA graph per main step. */
int g3m3_model_run(g3m3_model* m, int nsteps, int use_graph);
/* One main step from host state to host state.  `in` holds the state in
 * the g3m3_model_set_state layout (34 fields x n_grids x nz x ny x nx
 * floats); it is uploaded box by box, coarsest first, on a copy stream, and
 * the step waits for a box's upload only before it first touches that box,
 * so the finer boxes' uploads overlap the coarser boxes' steps.  After the
 * step (and the div B pass when one is due) the state is read back into
 * `out` (the same layout; it may be `in`).  With pinned buffers
 * (cudaMallocHost / cudaHostAlloc) the copies overlap as described and a
 * graph captured for a buffer is reused while the buffer stays the same;
 * pageable buffers are copied in and out around the step. */
int g3m3_model_step_host(g3m3_model* m, const float* in, float* out, int use_graph);
/* div B cleaning of every box plus flanks_synced and bndry_corer
 * (3d_main.f90:3363-3408). */
int g3m3_model_divb_all(g3m3_model* m);
/* Fluid (restart) files of the reference (3d_main.f90:3305-3349):
 * g3m3_model_write_fluid writes the current state, b0 and the inner-boundary
 * tables at the model's time t; g3m3_model_read_fluid loads them (cur and
 * wrk copies, b0, tables; the resistivity stays the model's) and sets t.
 * msrf/mmid/mzero are the table lengths the file was written with.  Call
 * g3m3_model_init_steps after reading, as for a fresh state. */
int g3m3_model_write_fluid(g3m3_model* m, const char* path);
int g3m3_model_read_fluid(g3m3_model* m, const char* path, int msrf,
    int mmid, int mzero);
/* Flux history (flux_counter, 3d_main.f90:1996-2011): from the next run
 * on, at the start of every main step the six fluxes of every box (boxes
 * n_grids..1, scaled by scale[box-1]) are recorded on the device, up to
 * `capacity` main steps; capacity 0 turns recording off.
 * g3m3_model_fluxes copies the history out: out[step][box-1][6] as
 * (q in, q out, h in, h out, o in, o out); *nsteps receives the steps
 * recorded. */
int g3m3_model_record_fluxes(g3m3_model* m, const float* scale, int capacity);
int g3m3_model_fluxes(g3m3_model* m, float* out, int* nsteps);
/* Graphing plane (sub_write_graphing_data.f90:340-420) of box `box` from
 * the current state: plane 0 = the x-y plane k = index, 1 = x-z at
 * j = index, 2 = y-z at i = index.  out[32][na][nb] (nb the faster grid
 * axis; x-y: ny x nx, x-z: nz x nx, y-z: nz x ny) holds, in code units:
 * 0-2 total B (b0 + b), 3 |B| (at least smallbit), 4-6 E (BandE), 7-9 J
 * (calcur); for species q, h, o in turn (10, 17, 24): velocity x, y, z
 * (p / max(rho, smallbit)), pressure parallel, perpendicular, cross
 * (fnd_pres), density; 31 electron pressure. */
int g3m3_model_graphing(g3m3_model* m, int box, int plane, int index,
    float* out);
/* Fresh-start state built on the device (3d_main.f90:1268-1629): dipole
 * background of strength alf_inner (moment along -z when negative),
 * corotating ionospheric plasma, the solar-wind fill from the params'
 * upstream values, the speed clip, a seeded multiplicative perturbation of
 * density and diagonal pressures (relative size `noise`, counter-based
 * normals from `seed`), the inner-boundary lists of boxes <= mbndry with
 * ionospheric densities scaled log-uniformly in [iono_lo, iono_hi], and the
 * resistivity shells.  Replaces g3m3_model_set_state/set_b0/set_inner for a
 * fresh start; call g3m3_model_init_steps next. */
int g3m3_model_init_state(g3m3_model* m, float alf_inner,
    unsigned long long seed, float noise, float iono_lo, float iono_hi);
/* Virtual spacecraft (cft_craft_handling.f90:120-200): ncraft <= 128
 * trajectories, craft c with npts[c] samples (x, y, z in planet radii, t in
 * the model's time units) sorted by t, all in traj(4, sum npts).  From the
 * next run on, at the end of every main step each craft's position at the
 * model time is interpolated between the samples around it (linterp,
 * cft_linterp.f90) and the fields `fields[0..nf-1]` (nf <= 8, indices of
 * g3m3_types.h) are sampled trilinearly in the smallest box holding it,
 * on the device, up to `capacity` steps; capacity 0 stops recording.
 * g3m3_model_craft_records copies out records [step][craft][4 + nf] =
 * (t, x, y, z, values); a craft whose trajectory does not cover t records
 * NaN. */
int g3m3_model_record_craft(g3m3_model* m, int ncraft, const int* npts,
    const float* traj, int nf, const int* fields, int capacity);
int g3m3_model_craft_records(g3m3_model* m, float* out, int* nsteps);
/* Tile shapes.  kernel 1 = fcsmooth: variant 0 = 32x8 tiles, 1 = 32x16,
 * 2 and 3 = 32x8 tiles with two fields per block in packed FP32x2
 * arithmetic, registers bounded for 3 or 4 resident blocks per SM; 4 and 5
 * = the two-field form with its planes copied asynchronously two plane
 * steps ahead and one barrier per plane (registers bounded for 3 or 2
 * blocks per SM); 6 = the same with the shortest rings (5 old/wrk slots,
 * 2 P1 slots: 55 KB) and 4 blocks per SM.
 * Every variant gives the same bits; only the speed differs.
 * g3m3_model_autotune times each variant on scratch copies of box 1 (the
 * state is not changed), keeps the fastest and reports it; cached step
 * graphs are dropped when the choice changes. */
#define G3M3_FCS_VARIANTS 8
int g3m3_model_set_variant(g3m3_model* m, int kernel, int variant);
/* The contracted flavour (on = 1): the push kernels built with fused
 * multiply-add contraction and quotients by a shared denominator taken as
 * products with its reciprocal.  Results are no longer the reference's FP32
 * bits; they stay within 1e-5 relative L2 per field per main step of them
 * (tests/test_contracted_gpu.py).  Off by default. */
int g3m3_model_set_contracted(g3m3_model* m, int on);
int g3m3_model_autotune(g3m3_model* m, int* fcs_variant);
/* Time bookkeeping: t, t_stepnew(1..n_grids), executed cell-updates. */
int g3m3_model_times(g3m3_model* m, double* t, double* t_stepnew,
    int64_t* cell_updates);
/* Graph mode captures a main step's graph the first time its plan (the
 * boxes' sub-cycling schedule and buffer roles) occurs, 20-30 ms once on the
 * production grid.  With n > 1 a plan runs host-launched (about 3 % slower
 * per step) until its n-th occurrence, so a schedule that occurs once in a
 * long run is never captured.  Default 1. */
int g3m3_model_set_capture_after(g3m3_model* m, int n);
/* The model's clock: the simulation time t and the main steps done, whose
 * count sets the div B cadence (a pass after every divb_every-th main
 * step).  Restoring a clock read before a run repeats the run's schedule of
 * div B passes from the same state. */
int g3m3_model_get_clock(g3m3_model* m, double* t, int* nsteps_done);
int g3m3_model_set_clock(g3m3_model* m, double t, int nsteps_done);
/* Launch counters of the last g3m3_model_run (kernels, graph launches). */
int g3m3_model_stats(g3m3_model* m, int64_t* kernels, int64_t* graphs);
/* Stream of the model (for CUDA-event timing by the caller). */
void* g3m3_model_stream(g3m3_model* m);
/* Measurement hook: launch one kernel of the engine `reps` times on box
 * `box` of the model, timed with CUDA events on the model's stream.
 * kernel: 0 push_ion (one species), 1 fcsmooth (34 fields), 2 set_rho +
 * set_speed_agrd pass, 3 Lapidus (one species, 10 fields), 4 flanks (34
 * fields, box < n_grids), 5 calcur + bs/btot, 6 BandE.  Outputs go to the
 * wrk/old copies, so call it only between runs whose state no longer
 * matters.  *bytes receives the algorithmic bytes of one launch. */
int g3m3_model_time_kernel(g3m3_model* m, int kernel, int box, int reps,
    float* ms_per_launch, double* bytes);

/* ---- ensembles ------------------------------------------------------
 * n independent states (params[0..n-1]; box sizes may differ, e.g. one
 * member per upstream condition) advanced together.  Each member is a
 * g3m3_model with its own CUDA stream, set up with the g3m3_model_* calls
 * through g3m3_ensemble_member (the ensemble owns and destroys it).
 * g3m3_ensemble_run advances every member by nsteps main steps: with
 * use_graph = 1, one main step of all members is one CUDA graph (members on
 * their own streams, overlapping on the GPU); 0, the members step one after
 * another from the host loop; 2, every member's kernels are launched from
 * the host on the member's own stream, all members at once; 3, every
 * member's own step graph (the one g3m3_model_run captures) is launched on
 * the member's own stream, all members at once.  Results are those of running each
 * member alone.  Work is ordered after earlier work on the ensemble's
 * stream (the context's) and before later work there. */
int g3m3_ensemble_create(g3m3_ctx* ctx, int n, const g3m3_params* params,
    g3m3_ensemble** out);
int g3m3_ensemble_destroy(g3m3_ensemble* e);
int g3m3_ensemble_member(g3m3_ensemble* e, int i, g3m3_model** out);
int g3m3_ensemble_run(g3m3_ensemble* e, int nsteps, int use_graph);
/* Kernels and graphs launched by the last run; cell-updates of all members. */
int g3m3_ensemble_stats(g3m3_ensemble* e, int64_t* kernels, int64_t* graphs,
    int64_t* cell_updates);
void* g3m3_ensemble_stream(g3m3_ensemble* e);

#ifdef __cplusplus
}
#endif
#endif
