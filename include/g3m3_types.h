/*
 * g3m3_types.h -- plain-C data types shared by the GB300 library
 * (include/g3m3.h) and its callers.
 *
 * Array convention (identical to the Fortran reference): every field is a
 * column-major FP32 array A(nx,ny,nz,n_grids) -- i fastest, then j, then k,
 * then box -- passed as a pointer to A(1,1,1,1).  Scratch fields of one box
 * are A(nx,ny,nz).  Index lists ijsrf(mbndry,3,msrf) etc. are int32
 * column-major.  Fortran logicals are int32, any nonzero value is .true.
 * (ifort writes -1, gfortran 1).
 */
#ifndef G3M3_TYPES_H
#define G3M3_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define G3M3_MAX_GRIDS 16
#define G3M3_NFIELDS 34

/* Field order used by every table in the library (the order of the
 * fluid-file records, 3d_main.f90:3310-3349): for species q, h, o the ten
 * fields rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz; then
 * epres, bx, by, bz. */
enum g3m3_field {
  G3M3_F_RHO = 0, G3M3_F_PX, G3M3_F_PY, G3M3_F_PZ,
  G3M3_F_PRESX, G3M3_F_PRESY, G3M3_F_PRESZ,
  G3M3_F_PRESXY, G3M3_F_PRESXZ, G3M3_F_PRESYZ,
  G3M3_SPECIES_FIELDS = 10,
  G3M3_F_EPRES = 30, G3M3_F_BX = 31, G3M3_F_BY = 32, G3M3_F_BZ = 33
};

/* Run constants.  One struct replaces the reference's namelist groups,
 * compile-time parameters and common blocks that the step reads
 * (3d_main.f90:54-72, 108-163, 582-602; common /rotation/). */
typedef struct g3m3_params {
  int32_t nx, ny, nz, n_grids;
  int32_t mbndry;            /* boxes 1..mbndry carry the inner boundary   */
  int32_t isotropic;         /* logical                                    */
  int32_t divb_every;        /* main steps between div B cleanings (0=off) */
  int32_t pad0;
  float xspac[G3M3_MAX_GRIDS];
  float grd_xmin[G3M3_MAX_GRIDS], grd_xmax[G3M3_MAX_GRIDS];
  float grd_ymin[G3M3_MAX_GRIDS], grd_ymax[G3M3_MAX_GRIDS];
  float grd_zmin[G3M3_MAX_GRIDS], grd_zmax[G3M3_MAX_GRIDS];
  /* species masses and fluid constants */
  float rmassq, rmassh, rmasso;
  float gamma, gamma1, reynolds, resist, grav, re_equiv;
  /* Lapidus (chi*) and flux-correction (dif*) coefficients */
  float chirho, chipxyz, chierg, difrho, diferg;
  /* guards: set_speed_agrd limits */
  float smallbit, aniso_limit, vlim_factor;
  float qvlim, hvlim, ovlim, qclim, hclim, oclim, cslim;
  /* time step control */
  float stepsz, t_step_max, t_step_min;
  /* solar wind at the inflow face (bndry_outer) */
  float srho, rho_frac, o_conc, spress, spx, spy, spz;
  float sbx_wind, sby_wind, sbz_wind, ti_te;
  /* inner boundary (bndry_inner) */
  float erho, epress, alpha_e, r_inner, v_rot, r_rot;
  /* div B cleaning */
  float divb_errlim;
  float pad1;
} g3m3_params;

#ifdef __cplusplus
}
#endif
#endif
