/*
 * g3m3_oracle.h -- CPU restatement of the G3M^3 multifluid time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle that the GB300 kernels are
 * checked against; nothing in the product links or calls it.  It restates,
 * statement for statement and in the reference's serial loop order, the
 * Fortran routines of itsmoosh/g3m3 (code/sub_*.f90, code/cft_*.f90 and the
 * step schedule of code/3d_main.f90).  Every function cites the reference
 * lines it follows.
 *
 * PINNED TO THE REFERENCE: the reference ships no tests, golden vectors or
 * fixtures (code/test.f90 is an empty stub) and is Fortran, for which the
 * build image has no compiler; oracle/fortran_to_c.py translates its own
 * routines and main loop to C (oracle/_ref, built from the sources where
 * they lie, never committed), and every routine here, the time-step set-up
 * and the main step agree with that build bitwise (tests/test_ref_pin.py,
 * tests/test_ref_main.py).  Analytic known-answer tests
 * (tests/test_oracle_kat.py) and the reference-made digests of
 * tests/golden/ hold it where the sources are absent.
 *
 * Conventions: arrays are column-major FP32 exactly as in the reference,
 * (nx,ny,nz,n_grids) with a 1-based box index, or (nx,ny,nz) for per-box
 * scratch.  Scalars that the Fortran passes by reference and only reads are
 * passed by value; scalars it writes are pointers.  Arithmetic is float with
 * the reference's operation order; build with -ffp-contract=off so that no
 * multiply-add is fused.
 */
#ifndef G3M3_ORACLE_H
#define G3M3_ORACLE_H

#include "../include/g3m3_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ----- a1-a3 pushes ---------------------------------------------------- */
void oracle_push_ion(
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

void oracle_push_elec(const float* wrkepres, const float* oldepres,
    float* epres, const float* evx, const float* evy, const float* evz,
    float gamma, float gamma1, int nx, int ny, int nz, int n_grids, int box,
    float delt, float rx, float ry, float rz);

void oracle_push_bfld(float* bx, float* by, float* bz,
    const float* oldbx, const float* oldby, const float* oldbz,
    const float* efldx, const float* efldy, const float* efldz,
    int nx, int ny, int nz, int n_grids, int box, float delt,
    float rx, float ry, float rz);

/* ----- a4-a6, a7 ------------------------------------------------------ */
void oracle_calcur(const float* bx, const float* by, const float* bz,
    int nx, int ny, int nz, int n_grids, int box,
    float* curx, float* cury, float* curz, float rx, float ry, float rz);

/* bs = b0 + b and btot = max(|bs|, smallbit) over one box
 * (3d_main.f90:2248-2254, 2491-2497). */
void oracle_total_b(const float* bx, const float* by, const float* bz,
    const float* bx0, const float* by0, const float* bz0,
    int nx, int ny, int nz, int n_grids, int box, float smallbit,
    float* bsx, float* bsy, float* bsz, float* btot);

void oracle_fnd_evel(const float* qpx, const float* qpy, const float* qpz,
    const float* qrho, const float* hpx, const float* hpy, const float* hpz,
    const float* hrho, const float* opx, const float* opy, const float* opz,
    const float* orho, const float* curx, const float* cury,
    const float* curz, float* evx, float* evy, float* evz,
    float* tvx, float* tvy, float* tvz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float reynolds);

void oracle_fnd_vtot(const float* qpx, const float* qpy, const float* qpz,
    const float* qrho, const float* hpx, const float* hpy, const float* hpz,
    const float* hrho, const float* opx, const float* opy, const float* opz,
    const float* orho, float* vx, float* vy, float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso);

void oracle_fnd_pres(const float* px, const float* py, const float* pz,
    const float* pxy, const float* pxz, const float* pyz,
    float* p_para, float* p_perp, float* p_cross,
    const float* vvx, const float* vvy, const float* vvz,
    const float* bxt, const float* byt, const float* bzt,
    int nx, int ny, int nz, int n_grids, int box);

void oracle_bande(float* efldx, float* efldy, float* efldz,
    const float* bsx, const float* bsy, const float* bsz,
    const float* curx, const float* cury, const float* curz,
    const float* evx, const float* evy, const float* evz, const float* btot,
    const float* epres, const float* qrho, const float* hrho,
    const float* orho, const float* rst, float resist, float reynolds,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso,
    const int* ijmid, const int* nummid, const int* ijzero, int mbndry,
    const int* numzero, int mmid, int mzero, float rx, float ry, float rz);

/* ----- a7-a9 smoothing ------------------------------------------------ */
void oracle_lap_plasma(const float* rho, const float* px, const float* py,
    const float* pz, const float* presx, const float* presy,
    const float* presz, const float* presxy, const float* presxz,
    const float* presyz,
    float* wrkrho, float* wrkpx, float* wrkpy, float* wrkpz,
    float* wrkpresx, float* wrkpresy, float* wrkpresz,
    float* wrkpresxy, float* wrkpresxz, float* wrkpresyz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt, int isotropic);

void oracle_lap_elec(const float* ppres, float* wrkppres,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt);

void oracle_lap_bfld(const float* bx, const float* by, const float* bz,
    float* wrkbx, float* wrkby, float* wrkbz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt);

void oracle_fcsmooth(float* px, const float* oldpx, const float* wrkpx,
    int nx, int ny, int nz, int n_grids, int box, float chipx,
    float* tempx, float* tempy, float* tempz);

/* flux_correct over the 34 fields given as pointer tables in the field order
 * of g3m3_types.h (sub_flux_correct.f90:107-189). */
void oracle_flux_correct(float* const cur[G3M3_NFIELDS],
    float* const wrk[G3M3_NFIELDS], float* const old[G3M3_NFIELDS],
    float* vvx, float* vvy, float* vvz,
    int nx, int ny, int nz, int n_grids, int box,
    float difrho, float diferg);

/* ----- a10-a12 guards -------------------------------------------------- */
void oracle_set_rho(float* qrho, float* qpresx, float* qpresy, float* qpresz,
    float* qpresxy, float* qpresxz, float* qpresyz, float rmassq,
    float* hrho, float* hpresx, float* hpresy, float* hpresz,
    float* hpresxy, float* hpresxz, float* hpresyz, float rmassh,
    float* orho, float* opresx, float* opresy, float* opresz,
    float* opresxy, float* opresxz, float* opresyz, float rmasso,
    float* epres, int nx, int ny, int nz, int n_grids, int box, float o_conc);

void oracle_set_speed_agrd(int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, int isotropic, float smallbit,
    float aniso_limit, float vlim, float qvlim, float hvlim, float ovlim,
    float qclim, float hclim, float oclim, float cslim,
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

void oracle_store_array(float* bx, const float* bx0,
    int nx, int ny, int nz, int n_grids, int box);

/* ----- a13-a17 boundaries and nested-grid sync ------------------------- */
/* bndry_outer over the 34 fields of box n_grids (sub_bndry_outer.f90). */
void oracle_bndry_outer(float* const f[G3M3_NFIELDS],
    const float* bx0, const float* by0, const float* bz0,
    const g3m3_params* p);

void oracle_bndry_inner(float* const f[G3M3_NFIELDS],
    const float* parm_srf, const float* parm_mid, const float* parm_zero,
    const int* ijsrf, const int* numsrf, const int* ijmid,
    const int* nummid, const int* ijzero, const int* numzero,
    int msrf, int mmid, int mzero, const g3m3_params* p);

void oracle_flanks(float* wrkrho, const float* rho, const float* oldrho,
    int nx, int ny, int nz, int n_grids, int box,
    const double* t_new, const double* t_old, double t, float* work,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax);

void oracle_corer(float* rho, int nx, int ny, int nz, int n_grids, int box,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax);

void oracle_flanks_synced(float* rho, int nx, int ny, int nz, int n_grids,
    int box, const float* grd_xmin, const float* grd_xmax,
    const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
    const float* grd_zmax);

/* ----- a18 div B ------------------------------------------------------- */
/* Returns the iteration count of the outermost CG loop; x0 = 0 (the
 * reference's soln_vec is uninitialised stack memory). */
/* sparse_solver (sub_sparse_solver.f90:19-159) on a caller's banded
 * matrix, right-hand side and starting iterate; returns the iterations of
 * the outermost call. */
int oracle_sparse_solver(int nbands, int npts, const int* divb_band_pos,
    float divb_errlim, int recurse, int redo_lim, const float* divb,
    float* soln_vec, float* residual2, float* banded_matrix);

int oracle_divb_correct(int nx, int ny, int nz, int n_grids, int box,
    int nbands, const int* divb_band_pos, const float* xspac,
    float divb_errlim, float* bx, float* by, float* bz);

/* ----- a19 virtual-spacecraft sampling -------------------------------- */
void oracle_findgrid(const float* xyz, int n_grids, const float* grid_minvals,
    const float* grid_maxvals, const float* xspac, int* gridpt,
    float re_equiv);
/* flux_counter (sub_flux_counter.f90:5-158) */
void oracle_flux_counter(const float* qpx, const float* qpy, const float* qpz,
    const float* hpx, const float* hpy, const float* hpz,
    const float* opx, const float* opy, const float* opz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float grid_spacing,
    float* qflux_in, float* qflux_out, float* hflux_in, float* hflux_out,
    float* oflux_in, float* oflux_out);

void oracle_trilin_interp(const float* sxyz, const float* gridpts,
    const float* qty, float* scdata);

/* ----- a20 the main step ---------------------------------------------- */
typedef struct oracle_state {
  float* cur[G3M3_NFIELDS];
  float* old[G3M3_NFIELDS];
  float* wrk[G3M3_NFIELDS];
  float* b0[3];
  float* resistive;                 /* (nx,ny,nz,mbndry) */
  int *ijsrf, *ijmid, *ijzero;      /* (mbndry,3,m*)     */
  int *numsrf, *nummid, *numzero;   /* (mbndry)          */
  float *parm_srf, *parm_mid, *parm_zero;  /* (mbndry,7,m*) */
  int msrf, mmid, mzero;
  /* one-box scratch (nx,ny,nz) */
  float *efld[3], *curr[3], *bs[3], *btot, *vv[3], *tv[3], *ev[3];
  double t;
  double t_old[G3M3_MAX_GRIDS], t_new[G3M3_MAX_GRIDS];
  double t_step[G3M3_MAX_GRIDS], t_stepnew[G3M3_MAX_GRIDS];
  int64_t cell_updates;             /* executed box-steps x cells */
  int32_t nsteps_done;
  int32_t last_cg_iters;
} oracle_state;

/* Initial guards and time steps: the "Check initial conditions" loop,
 * 3d_main.f90:1861-1903. */
void oracle_init_steps(const g3m3_params* p, oracle_state* s);

/* One iteration of the main time loop, 3d_main.f90:1925-3095 (without the
 * flux counter, graph dump, torus injection and file output).  Returns 0,
 * or 1 when the step fell below t_step_min (the reference stops). */
int oracle_main_step(const g3m3_params* p, oracle_state* s);

/* div B cleaning of all boxes followed by flanks_synced and bndry_corer,
 * 3d_main.f90:1067-1123 / 3363-3408. */
void oracle_divb_all(const g3m3_params* p, oracle_state* s);

#ifdef __cplusplus
}
#endif
#endif
