/*
 * g3m3_oracle_kernels.c -- TEST INFRASTRUCTURE: CPU restatement of the
 * per-box routines of the G3M^3 step (reference rows a1-a19).  Only the test
 * suite, the smoke check and bench.py's CPU-baseline leg use it.
 *
 * Pinned bitwise to the reference's own routines, translated from its
 * Fortran and compiled (see g3m3_oracle.h).  Each function follows the cited Fortran statement for
 * statement; float literals keep every operation in FP32 and the operand
 * order of the source is kept.  Loops whose iterations are independent carry
 * an OpenMP pragma: with or without -fopenmp they give identical bits.
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include "g3m3_oracle.h"

#define IX(i, j, k) \
  ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))
#define BOXP(a) ((a) + (size_t)(box - 1) * (size_t)nx * (size_t)ny * (size_t)nz)

static inline float amax1(float a, float b) { return a > b ? a : b; }
static inline float amin1(float a, float b) { return a < b ? a : b; }
/* ifort SIGN(1.,x) with its default -assume nominus0: +1 for x = -0. */
static inline float sign1(float x) { return x >= 0.0f ? 1.0f : -1.0f; }

/* ======================================================================
 * push_ion -- sub_push_ion.f90:4-362
 * ==================================================================== */
void oracle_push_ion(
    float* qrho_, float* qpresx_, float* qpresy_, float* qpresz_,
    float* qpx_, float* qpy_, float* qpz_,
    const float* oldqrho_, const float* oldqpresx_, const float* oldqpresy_,
    const float* oldqpresz_, const float* oldqpx_, const float* oldqpy_,
    const float* oldqpz_,
    const float* wrkqrho_, const float* wrkqpresx_, const float* wrkqpresy_,
    const float* wrkqpresz_, const float* wrkqpx_, const float* wrkqpy_,
    const float* wrkqpz_,
    float* qpresxy_, float* qpresxz_, float* qpresyz_,
    const float* oldqpresxy_, const float* oldqpresxz_,
    const float* oldqpresyz_,
    const float* wrkqpresxy_, const float* wrkqpresxz_,
    const float* wrkqpresyz_,
    const float* bsx, const float* bsy, const float* bsz, const float* btot,
    const float* efldx, const float* efldy, const float* efldz, float rmassq,
    float* qvx, float* qvy, float* qvz,
    const float* tvx, const float* tvy, const float* tvz,
    float gamma, float gamma1,
    int nx, int ny, int nz, int n_grids, int box, float delt, float grav,
    float re_equiv, float reynolds,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax,
    int isotropic) {
  (void)gamma; (void)gamma1; (void)n_grids; (void)isotropic;
  float* qrho = BOXP(qrho_); float* qpresx = BOXP(qpresx_);
  float* qpresy = BOXP(qpresy_); float* qpresz = BOXP(qpresz_);
  float* qpx = BOXP(qpx_); float* qpy = BOXP(qpy_); float* qpz = BOXP(qpz_);
  float* qpresxy = BOXP(qpresxy_); float* qpresxz = BOXP(qpresxz_);
  float* qpresyz = BOXP(qpresyz_);
  const float* oldqrho = BOXP(oldqrho_); const float* oldqpresx = BOXP(oldqpresx_);
  const float* oldqpresy = BOXP(oldqpresy_); const float* oldqpresz = BOXP(oldqpresz_);
  const float* oldqpx = BOXP(oldqpx_); const float* oldqpy = BOXP(oldqpy_);
  const float* oldqpz = BOXP(oldqpz_);
  const float* oldqpresxy = BOXP(oldqpresxy_); const float* oldqpresxz = BOXP(oldqpresxz_);
  const float* oldqpresyz = BOXP(oldqpresyz_);
  const float* wrkqrho = BOXP(wrkqrho_); const float* wrkqpresx = BOXP(wrkqpresx_);
  const float* wrkqpresy = BOXP(wrkqpresy_); const float* wrkqpresz = BOXP(wrkqpresz_);
  const float* wrkqpx = BOXP(wrkqpx_); const float* wrkqpy = BOXP(wrkqpy_);
  const float* wrkqpz = BOXP(wrkqpz_);
  const float* wrkqpresxy = BOXP(wrkqpresxy_); const float* wrkqpresxz = BOXP(wrkqpresxz_);
  const float* wrkqpresyz = BOXP(wrkqpresyz_);

  /* :50-64 */
  const float ddx = (grd_xmax[box - 1] - grd_xmin[box - 1]) / (float)(nx - 1);
  const float ddy = (grd_ymax[box - 1] - grd_ymin[box - 1]) / (float)(ny - 1);
  const float ddz = (grd_zmax[box - 1] - grd_zmin[box - 1]) / (float)(nz - 1);
  const float dxt = 2.0f * ddx, dyt = 2.0f * ddy, dzt = 2.0f * ddz;
  const float d_min = 1.e-6f;
  const float rmass = rmassq;
  const float bmax = 0.20f * rmassq / delt / reynolds;

  /* velocity pre-pass :67-81 */
#pragma omp parallel for
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        size_t c = IX(i, j, k);
        float aqrho = amax1(wrkqrho[c], d_min);
        qvx[c] = wrkqpx[c] / aqrho;
        qvy[c] = wrkqpy[c] / aqrho;
        qvz[c] = wrkqpz[c] / aqrho;
      }

  /* stencil loop :87-359 */
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++) {
    const int km = k - 1, kk = k + 1;
    const float az = grd_zmin[box - 1] + ddz * (float)(k - 1);
    for (int j = 2; j <= ny - 1; j++) {
      const int jm = j - 1, jj = j + 1;
      const float ay = grd_ymin[box - 1] + ddy * (float)(j - 1);
      for (int i = 2; i <= nx - 1; i++) {
        const float ax = grd_xmin[box - 1] + ddx * (float)(i - 1);
        const int ii = i + 1, im = i - 1;
        const size_t c = IX(i, j, k);
        const size_t xp = IX(ii, j, k), xm = IX(im, j, k);
        const size_t yp = IX(i, jj, k), ym = IX(i, jm, k);
        const size_t zp = IX(i, j, kk), zm = IX(i, j, km);

        /* continuity :107-110 */
        qrho[c] = oldqrho[c] - delt * (((wrkqpx[xp] - wrkqpx[xm]) / dxt)
                                       + ((wrkqpy[yp] - wrkqpy[ym]) / dyt)
                                       + ((wrkqpz[zp] - wrkqpz[zm]) / dzt));
        /* momentum fluxes :112-134 */
        float aqpx = oldqpx[c] - delt * (((wrkqpx[xp] * qvx[xp] - wrkqpx[xm] * qvx[xm]) / dxt)
                                         + ((wrkqpx[yp] * qvy[yp] - wrkqpx[ym] * qvy[ym]) / dyt)
                                         + ((wrkqpx[zp] * qvz[zp] - wrkqpx[zm] * qvz[zm]) / dzt));
        float aqpy = oldqpy[c] - delt * (((wrkqpy[xp] * qvx[xp] - wrkqpy[xm] * qvx[xm]) / dxt)
                                         + ((wrkqpy[yp] * qvy[yp] - wrkqpy[ym] * qvy[ym]) / dyt)
                                         + ((wrkqpy[zp] * qvz[zp] - wrkqpy[zm] * qvz[zm]) / dzt));
        float aqpz = oldqpz[c] - delt * (((wrkqpz[xp] * qvx[xp] - wrkqpz[xm] * qvx[xm]) / dxt)
                                         + ((wrkqpz[yp] * qvy[yp] - wrkqpz[ym] * qvy[ym]) / dyt)
                                         + ((wrkqpz[zp] * qvz[zp] - wrkqpz[zm] * qvz[zm]) / dzt));
        /* :138-143 */
        float abx = bsx[c], aby = bsy[c], abz = bsz[c];
        float bmag = btot[c];
        float weight = amax1(1.0f, bmag / bmax);
        float skin_depth = reynolds / weight;
        /* :145-151 */
        float tvcrossb_x = (tvy[c] * abz - tvz[c] * aby);
        float tvcrossb_y = -(tvx[c] * abz - tvz[c] * abx);
        float tvcrossb_z = (tvx[c] * aby - tvy[c] * abx);
        float qvcrossb_x = (qvy[c] * abz - qvz[c] * aby);
        float qvcrossb_y = -(qvx[c] * abz - qvz[c] * abx);
        float qvcrossb_z = (qvx[c] * aby - qvy[c] * abx);
        /* pressure gradient :153-170 (dxt used for some y/z terms, as in
         * the reference) */
        float qgradp_x = (wrkqpresx[xp] - wrkqpresx[xm]) / dxt
                         + (wrkqpresxy[yp] - wrkqpresxy[ym]) / dxt
                         + (wrkqpresxz[zp] - wrkqpresxz[zm]) / dxt;
        float qgradp_y = (wrkqpresxy[xp] - wrkqpresxy[xm]) / dxt
                         + (wrkqpresy[yp] - wrkqpresy[ym]) / dyt
                         + (wrkqpresyz[zp] - wrkqpresyz[zm]) / dxt;
        float qgradp_z = (wrkqpresxz[xp] - wrkqpresxz[xm]) / dxt
                         + (wrkqpresyz[yp] - wrkqpresyz[ym]) / dyt
                         + (wrkqpresz[zp] - wrkqpresz[zm]) / dzt;
        /* :174-188 */
        float dele_x = (efldx[c] + tvcrossb_x) * reynolds;
        float dele_y = (efldy[c] + tvcrossb_y) * reynolds;
        float dele_z = (efldz[c] + tvcrossb_z) * reynolds;
        float delv_x = (qvcrossb_x - tvcrossb_x) * skin_depth;
        float delv_y = (qvcrossb_y - tvcrossb_y) * skin_depth;
        float delv_z = (qvcrossb_z - tvcrossb_z) * skin_depth;
        float qden = wrkqrho[c] / rmassq;
        float npx = aqpx + delt * (qden * (dele_x + delv_x) - qgradp_x);
        float npy = aqpy + delt * (qden * (dele_y + delv_y) - qgradp_y);
        float npz = aqpz + delt * (qden * (dele_z + delv_z) - qgradp_z);
        /* gravity :202-206 */
        float radius = sqrtf(ax * ax + ay * ay + az * az) + 0.0000001f;
        float rr = re_equiv * radius;
        float g = delt * wrkqrho[c] * grav / (rr * rr);
        qpx[c] = npx - g * ax / radius;
        qpy[c] = npy - g * ay / radius;
        qpz[c] = npz - g * az / radius;

        /* diagonal pressures :210-238 */
        float px_ = oldqpresx[c] - delt * (((wrkqpresx[xp] * qvx[xp] - wrkqpresx[xm] * qvx[xm]) / dxt)
                                           + ((wrkqpresx[yp] * qvy[yp] - wrkqpresx[ym] * qvy[ym]) / dyt)
                                           + ((wrkqpresx[zp] * qvz[zp] - wrkqpresx[zm] * qvz[zm]) / dzt))
                    - 2.0f * delt * wrkqpresx[c] * (qvx[xp] - qvx[xm]) / dxt;
        float py_ = oldqpresy[c] - delt * (((wrkqpresy[xp] * qvx[xp] - wrkqpresy[xm] * qvx[xm]) / dxt)
                                           + ((wrkqpresy[yp] * qvy[yp] - wrkqpresy[ym] * qvy[ym]) / dyt)
                                           + ((wrkqpresy[zp] * qvz[zp] - wrkqpresy[zm] * qvz[zm]) / dzt))
                    - 2.0f * delt * wrkqpresy[c] * (qvy[yp] - qvy[ym]) / dyt;
        float pz_ = oldqpresz[c] - delt * (((wrkqpresz[xp] * qvx[xp] - wrkqpresz[xm] * qvx[xm]) / dxt)
                                           + ((wrkqpresz[yp] * qvy[yp] - wrkqpresz[ym] * qvy[ym]) / dyt)
                                           + ((wrkqpresz[zp] * qvz[zp] - wrkqpresz[zm] * qvz[zm]) / dzt))
                    - 2.0f * delt * wrkqpresz[c] * (qvz[zp] - qvz[zm]) / dzt;

        /* 12-point smoothed B for the gyro term :242-254 */
        abx = (6.0f * bsx[c] + bsx[xp] + bsx[xm] + bsx[yp] + bsx[ym] + bsx[zp] + bsx[zm]) / 12.0f;
        aby = (6.0f * bsy[c] + bsy[xp] + bsy[xm] + bsy[yp] + bsy[ym] + bsy[zp] + bsy[zm]) / 12.0f;
        abz = (6.0f * bsz[c] + bsz[xp] + bsz[xm] + bsz[yp] + bsz[ym] + bsz[zp] + bsz[zm]) / 12.0f;
        bmag = sqrtf(abx * abx + aby * aby + abz * abz);
        float skin_factor = reynolds;
        if (bmag > bmax) skin_factor = reynolds * (bmax / bmag);

        const float wxy = wrkqpresxy[c], wxz = wrkqpresxz[c], wyz = wrkqpresyz[c];
        const float wx = wrkqpresx[c], wy = wrkqpresy[c], wz = wrkqpresz[c];
        /* anisotropic diagonal terms :256-281 */
        qpresx[c] = px_ - 2.0f * delt * wxy * (qvx[yp] - qvx[ym]) / dyt
                    - 2.0f * delt * wxz * (qvx[zp] - qvx[zm]) / dzt
                    + 2.0f * delt * skin_factor / rmass * (wxy * abz - wxz * aby);
        qpresy[c] = py_ - 2.0f * delt * wxy * (qvy[xp] - qvy[xm]) / dxt
                    - 2.0f * delt * wyz * (qvy[zp] - qvy[zm]) / dzt
                    + 2.0f * delt * skin_factor / rmass * (wyz * abx - wxy * abz);
        qpresz[c] = pz_ - 2.0f * delt * wxz * (qvz[xp] - qvz[xm]) / dxt
                    - 2.0f * delt * wyz * (qvz[yp] - qvz[ym]) / dyt
                    + 2.0f * delt * skin_factor / rmass * (wxz * aby - wyz * abx);

        /* off-diagonal elements :285-356 */
        float pxy = oldqpresxy[c] - delt * (((wrkqpresxy[xp] * qvx[xp] - wrkqpresxy[xm] * qvx[xm]) / dxt)
                                            + ((wrkqpresxy[yp] * qvy[yp] - wrkqpresxy[ym] * qvy[ym]) / dyt)
                                            + ((wrkqpresxy[zp] * qvz[zp] - wrkqpresxy[zm] * qvz[zm]) / dzt));
        qpresxy[c] = pxy - delt * wxy * ((qvx[xp] - qvx[xm]) / dxt + (qvy[yp] - qvy[ym]) / dyt)
                     - delt * wy * (qvx[yp] - qvx[ym]) / dyt
                     - delt * wx * (qvy[xp] - qvy[xm]) / dxt
                     - delt * wyz * (qvx[zp] - qvx[zm]) / dzt
                     - delt * wxz * (qvy[zp] - qvy[zm]) / dzt
                     + delt * skin_factor / rmass * (abz * (wy - wx) - aby * wyz + abx * wxz);

        float pxz = oldqpresxz[c] - delt * (((wrkqpresxz[xp] * qvx[xp] - wrkqpresxz[xm] * qvx[xm]) / dxt)
                                            + ((wrkqpresxz[yp] * qvy[yp] - wrkqpresxz[ym] * qvy[ym]) / dyt)
                                            + ((wrkqpresxz[zp] * qvz[zp] - wrkqpresxz[zm] * qvz[zm]) / dzt));
        qpresxz[c] = pxz - delt * wxz * ((qvx[xp] - qvx[xm]) / dxt + (qvz[zp] - qvz[zm]) / dzt)
                     - delt * wz * (qvx[zp] - qvx[zm]) / dzt
                     - delt * wx * (qvz[xp] - qvz[xm]) / dxt
                     - delt * wyz * (qvx[yp] - qvx[ym]) / dyt
                     - delt * wxy * (qvz[yp] - qvz[ym]) / dyt
                     + delt * skin_factor / rmass * (aby * (wx - wz) - abx * wxy + abz * wyz);

        float pyz = oldqpresyz[c] - delt * (((wrkqpresyz[xp] * qvx[xp] - wrkqpresyz[xm] * qvx[xm]) / dxt)
                                            + ((wrkqpresyz[yp] * qvy[yp] - wrkqpresyz[ym] * qvy[ym]) / dyt)
                                            + ((wrkqpresyz[zp] * qvz[zp] - wrkqpresyz[zm] * qvz[zm]) / dzt));
        qpresyz[c] = pyz - delt * wyz * ((qvy[yp] - qvy[ym]) / dyt + (qvz[zp] - qvz[zm]) / dzt)
                     - delt * wy * (qvz[yp] - qvz[ym]) / dyt
                     - delt * wz * (qvy[zp] - qvy[zm]) / dzt
                     - delt * wxy * (qvz[xp] - qvz[xm]) / dxt
                     - delt * wxz * (qvy[xp] - qvy[xm]) / dxt
                     + delt * skin_factor / rmass * (abx * (wz - wy) - abz * wxz + aby * wxy);
      }
    }
  }
}

/* ======================================================================
 * push_elec -- sub_push_elec.f90:4-53 (reads arg 1, writes arg 3)
 * ==================================================================== */
void oracle_push_elec(const float* wrkepres_, const float* oldepres_,
    float* epres_, const float* evx, const float* evy, const float* evz,
    float gamma, float gamma1, int nx, int ny, int nz, int n_grids, int box,
    float delt, float rx, float ry, float rz) {
  (void)n_grids;
  const float* wrkepres = BOXP(wrkepres_);
  const float* oldepres = BOXP(oldepres_);
  float* epres = BOXP(epres_);
  const float dxt = 2.0f * rx, dyt = 2.0f * ry, dzt = 2.0f * rz;
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        const size_t xp = IX(i + 1, j, k), xm = IX(i - 1, j, k);
        const size_t yp = IX(i, j + 1, k), ym = IX(i, j - 1, k);
        const size_t zp = IX(i, j, k + 1), zm = IX(i, j, k - 1);
        float egradp_x = (wrkepres[xp] - wrkepres[xm]) / dxt;
        float egradp_y = (wrkepres[yp] - wrkepres[ym]) / dyt;
        float egradp_z = (wrkepres[zp] - wrkepres[zm]) / dzt;
        float e = oldepres[c] - delt * gamma * (((wrkepres[xp] * evx[xp] - wrkepres[xm] * evx[xm]) / dxt)
                                                + ((wrkepres[yp] * evy[yp] - wrkepres[ym] * evy[ym]) / dyt)
                                                + ((wrkepres[zp] * evz[zp] - wrkepres[zm] * evz[zm]) / dzt));
        epres[c] = e + delt * gamma1 * (evx[c] * egradp_x + evy[c] * egradp_y + evz[c] * egradp_z);
      }
}

/* ======================================================================
 * push_bfld -- sub_push_bfld.f90:4-50
 * ==================================================================== */
void oracle_push_bfld(float* bx_, float* by_, float* bz_,
    const float* oldbx_, const float* oldby_, const float* oldbz_,
    const float* efldx, const float* efldy, const float* efldz,
    int nx, int ny, int nz, int n_grids, int box, float delt,
    float rx, float ry, float rz) {
  (void)n_grids;
  float* bx = BOXP(bx_); float* by = BOXP(by_); float* bz = BOXP(bz_);
  const float* oldbx = BOXP(oldbx_); const float* oldby = BOXP(oldby_);
  const float* oldbz = BOXP(oldbz_);
  const float dxt = 2.0f * rx, dyt = 2.0f * ry, dzt = 2.0f * rz;
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        const size_t xp = IX(i + 1, j, k), xm = IX(i - 1, j, k);
        const size_t yp = IX(i, j + 1, k), ym = IX(i, j - 1, k);
        const size_t zp = IX(i, j, k + 1), zm = IX(i, j, k - 1);
        bx[c] = oldbx[c] - delt * (((efldz[yp] - efldz[ym]) / dyt) - ((efldy[zp] - efldy[zm]) / dzt));
        by[c] = oldby[c] + delt * (((efldz[xp] - efldz[xm]) / dxt) - ((efldx[zp] - efldx[zm]) / dzt));
        bz[c] = oldbz[c] - delt * (((efldy[xp] - efldy[xm]) / dxt) - ((efldx[yp] - efldx[ym]) / dyt));
      }
}

/* ======================================================================
 * calcur -- sub_calcur.f90:5-189
 * ==================================================================== */
void oracle_calcur(const float* bx_, const float* by_, const float* bz_,
    int nx, int ny, int nz, int n_grids, int box,
    float* curx, float* cury, float* curz, float rx, float ry, float rz) {
  (void)n_grids;
  const float* bx = BOXP(bx_); const float* by = BOXP(by_); const float* bz = BOXP(bz_);
  const float dxt = 2.0f * rx, dyt = 2.0f * ry, dzt = 2.0f * rz;
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        curx[c] = (bz[IX(i, j + 1, k)] - bz[IX(i, j - 1, k)]) / dyt
                  - (by[IX(i, j, k + 1)] - by[IX(i, j, k - 1)]) / dzt;
        cury[c] = (bx[IX(i, j, k + 1)] - bx[IX(i, j, k - 1)]) / dzt
                  - (bz[IX(i + 1, j, k)] - bz[IX(i - 1, j, k)]) / dxt;
        curz[c] = (by[IX(i + 1, j, k)] - by[IX(i - 1, j, k)]) / dxt
                  - (bx[IX(i, j + 1, k)] - bx[IX(i, j - 1, k)]) / dyt;
      }
  const int nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;
  float* cc[3] = {curx, cury, curz};
  for (int q = 0; q < 3; q++) {
    float* c = cc[q];
    /* bottom and top panels :224-238 */
    for (int j = 2; j <= ny1; j++)
      for (int i = 2; i <= nx1; i++) {
        c[IX(i, j, 1)] = c[IX(i, j, 2)];
        c[IX(i, j, nz)] = c[IX(i, j, nz1)];
      }
    /* front and back :243-255 */
    for (int k = 2; k <= nz1; k++)
      for (int j = 2; j <= ny1; j++) {
        c[IX(1, j, k)] = c[IX(2, j, k)];
        c[IX(nx, j, k)] = c[IX(nx1, j, k)];
      }
    /* left and right :260-271 (the loop variable j runs over z) */
    for (int k = 2; k <= nz1; k++)
      for (int i = 2; i <= nx1; i++) {
        c[IX(i, 1, k)] = c[IX(i, 2, k)];
        c[IX(i, ny, k)] = c[IX(i, ny1, k)];
      }
    /* corner lines :276-324 */
    for (int i = 2; i <= nx1; i++) {
      c[IX(i, 1, 1)] = c[IX(i, 1, 2)];
      c[IX(i, 1, nz)] = c[IX(i, 1, nz1)];
      c[IX(i, ny, 1)] = c[IX(i, ny, 2)];
      c[IX(i, ny, nz)] = c[IX(i, ny1, nz)];
    }
    for (int j = 2; j <= ny1; j++) {
      c[IX(1, j, 1)] = c[IX(1, j, 2)];
      c[IX(1, j, nz)] = c[IX(1, j, nz1)];
      c[IX(nx, j, 1)] = c[IX(nx, j, 2)];
      c[IX(nx, j, nz)] = c[IX(nx, j, nz1)];
    }
    for (int k = 2; k <= nz1; k++) {
      c[IX(1, 1, k)] = c[IX(1, 2, k)];
      c[IX(nx, 1, k)] = c[IX(nx, 2, k)];
      c[IX(1, ny, k)] = c[IX(1, ny1, k)];
      c[IX(nx, ny, k)] = c[IX(nx, ny1, k)];
    }
    /* corners :326-351 */
    c[IX(1, 1, 1)] = c[IX(1, 1, 2)];
    c[IX(1, ny, 1)] = c[IX(1, ny, 2)];
    c[IX(1, 1, nz)] = (c[IX(1, 1, nz1)] + c[IX(1, 2, nz)]) / 2.0f;
    c[IX(1, ny, nz)] = (c[IX(1, ny, nz1)] + c[IX(1, ny1, nz)]) / 2.0f;
    c[IX(nx, 1, 1)] = (c[IX(nx, 1, 2)] + c[IX(nx, 2, 1)] + c[IX(nx1, 1, 1)]) / 3.0f;
    c[IX(nx, ny, 1)] = (c[IX(nx, ny, 2)] + c[IX(nx, ny1, 1)] + c[IX(nx1, ny, 1)]) / 3.0f;
    c[IX(nx, 1, nz)] = (c[IX(nx, 1, nz1)] + c[IX(nx, 2, nz)] + c[IX(nx1, 1, nz)]) / 3.0f;
    c[IX(nx, ny, nz)] = (c[IX(nx, ny, nz1)] + c[IX(nx, ny1, nz)] + c[IX(nx1, ny, nz)]) / 3.0f;
  }
}

void oracle_total_b(const float* bx_, const float* by_, const float* bz_,
    const float* bx0_, const float* by0_, const float* bz0_,
    int nx, int ny, int nz, int n_grids, int box, float smallbit,
    float* bsx, float* bsy, float* bsz, float* btot) {
  (void)n_grids;
  const float* bx = BOXP(bx_); const float* by = BOXP(by_); const float* bz = BOXP(bz_);
  const float* bx0 = BOXP(bx0_); const float* by0 = BOXP(by0_); const float* bz0 = BOXP(bz0_);
  const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    bsx[c] = bx0[c] + bx[c];
    bsy[c] = by0[c] + by[c];
    bsz[c] = bz0[c] + bz[c];
    btot[c] = amax1(sqrtf(bsx[c] * bsx[c] + bsy[c] * bsy[c] + bsz[c] * bsz[c]), smallbit);
  }
}

/* ======================================================================
 * fnd_evel -- sub_fnd_evel.f90:4-57
 * ==================================================================== */
void oracle_fnd_evel(const float* qpx_, const float* qpy_, const float* qpz_,
    const float* qrho_, const float* hpx_, const float* hpy_,
    const float* hpz_, const float* hrho_, const float* opx_,
    const float* opy_, const float* opz_, const float* orho_,
    const float* curx, const float* cury, const float* curz,
    float* evx, float* evy, float* evz, float* tvx, float* tvy, float* tvz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float reynolds) {
  (void)n_grids;
  const float *qpx = BOXP(qpx_), *qpy = BOXP(qpy_), *qpz = BOXP(qpz_), *qrho = BOXP(qrho_);
  const float *hpx = BOXP(hpx_), *hpy = BOXP(hpy_), *hpz = BOXP(hpz_), *hrho = BOXP(hrho_);
  const float *opx = BOXP(opx_), *opy = BOXP(opy_), *opz = BOXP(opz_), *orho = BOXP(orho_);
  const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    float qden = (qrho[c] + 0.000001f) / rmassq;
    float hden = (hrho[c] + 0.000001f) / rmassh;
    float oden = (orho[c] + 0.000001f) / rmasso;
    float tot_numden = qden + hden + oden;
    float tden = qrho[c] + hrho[c] + orho[c];
    tvx[c] = (qpx[c] + hpx[c] + opx[c]) / tden;
    evx[c] = tvx[c] - curx[c] / tot_numden / reynolds;
    tvy[c] = (qpy[c] + hpy[c] + opy[c]) / tden;
    evy[c] = tvy[c] - cury[c] / tot_numden / reynolds;
    tvz[c] = (qpz[c] + hpz[c] + opz[c]) / tden;
    evz[c] = tvz[c] - curz[c] / tot_numden / reynolds;
  }
}

/* fnd_vtot -- sub_fnd_vtot.f90:4-41 */
void oracle_fnd_vtot(const float* qpx_, const float* qpy_, const float* qpz_,
    const float* qrho_, const float* hpx_, const float* hpy_,
    const float* hpz_, const float* hrho_, const float* opx_,
    const float* opy_, const float* opz_, const float* orho_,
    float* vx, float* vy, float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso) {
  (void)n_grids; (void)rmassq; (void)rmassh; (void)rmasso;
  const float *qpx = BOXP(qpx_), *qpy = BOXP(qpy_), *qpz = BOXP(qpz_), *qrho = BOXP(qrho_);
  const float *hpx = BOXP(hpx_), *hpy = BOXP(hpy_), *hpz = BOXP(hpz_), *hrho = BOXP(hrho_);
  const float *opx = BOXP(opx_), *opy = BOXP(opy_), *opz = BOXP(opz_), *orho = BOXP(orho_);
  const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    float tden = qrho[c] + hrho[c] + orho[c];
    vx[c] = (qpx[c] + hpx[c] + opx[c]) / tden;
    vy[c] = (qpy[c] + hpy[c] + opy[c]) / tden;
    vz[c] = (qpz[c] + hpz[c] + opz[c]) / tden;
  }
}

/* fnd_pres -- sub_fnd_pres.f90:5-67 */
void oracle_fnd_pres(const float* px_, const float* py_, const float* pz_,
    const float* pxy_, const float* pxz_, const float* pyz_,
    float* p_para_, float* p_perp_, float* p_cross_,
    const float* vvx, const float* vvy, const float* vvz,
    const float* bxt, const float* byt, const float* bzt,
    int nx, int ny, int nz, int n_grids, int box) {
  (void)n_grids; (void)pxy_; (void)pxz_; (void)pyz_;
  const float *px = BOXP(px_), *py = BOXP(py_), *pz = BOXP(pz_);
  float *p_para = BOXP(p_para_), *p_perp = BOXP(p_perp_), *p_cross = BOXP(p_cross_);
  const size_t n = (size_t)nx * ny * nz;
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    float presx = px[c], presy = py[c], presz = pz[c];
    float presmag = sqrtf(presx * presx + presy * presy + presz * presz) + 1.e-11f;
    float abx = bxt[c], aby = byt[c], abz = bzt[c];
    float bmag = sqrtf(abx * abx + aby * aby + abz * abz) + 1.e-12f;
    float avx = vvx[c], avy = vvy[c], avz = vvz[c];
    float vcbx = (avy * abz - avz * aby) / bmag;
    float vcby = -(avx * abz - avz * abx) / bmag;
    float vcbz = (avx * aby - avy * abx) / bmag;
    float vcmag = sqrtf(vcbx * vcbx + vcby * vcby + vcbz * vcbz) + 1.e-12f;
    float a1 = abx * presx, a2 = aby * presy, a3 = abz * presz;
    float para = sqrtf(a1 * a1 + a2 * a2 + a3 * a3) / bmag;
    float b1 = vcbx * presx, b2 = vcby * presy, b3 = vcbz * presz;
    float cross = sqrtf(b1 * b1 + b2 * b2 + b3 * b3) / vcmag;
    p_para[c] = para;
    p_cross[c] = cross;
    p_perp[c] = sqrtf(fabsf(presmag * presmag - (para * para + cross * cross)));
  }
}

/* ======================================================================
 * BandE -- sub_BandE.f90:5-162
 * ==================================================================== */
void oracle_bande(float* efldx, float* efldy, float* efldz,
    const float* bsx, const float* bsy, const float* bsz,
    const float* curx, const float* cury, const float* curz,
    const float* evx, const float* evy, const float* evz, const float* btot,
    const float* epres_, const float* qrho_, const float* hrho_,
    const float* orho_, const float* rst_, float resist, float reynolds,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso,
    const int* ijmid, const int* nummid, const int* ijzero, int mbndry,
    const int* numzero, int mmid, int mzero, float rx, float ry, float rz) {
  (void)n_grids; (void)btot;
  const float *epres = BOXP(epres_), *qrho = BOXP(qrho_), *hrho = BOXP(hrho_), *orho = BOXP(orho_);
  const size_t n = (size_t)nx * ny * nz;
  /* Ohm's law :32-51 */
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    float avx = evx[c], avy = evy[c], avz = evz[c];
    float abx = bsx[c], aby = bsy[c], abz = bsz[c];
    efldx[c] = -(avy * abz - avz * aby);
    efldy[c] = -(avz * abx - avx * abz);
    efldz[c] = -(avx * aby - avy * abx);
  }
  /* grad p_e :55-84 */
  const float dxt = 2.0f * rx, dyt = 2.0f * ry, dzt = 2.0f * rz;
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        float arho = (qrho[c] / rmassq + hrho[c] / rmassh + orho[c] / rmasso) * reynolds;
        efldx[c] = efldx[c] - ((epres[IX(i + 1, j, k)] - epres[IX(i - 1, j, k)]) / dxt) / arho;
        efldy[c] = efldy[c] - ((epres[IX(i, j + 1, k)] - epres[IX(i, j - 1, k)]) / dyt) / arho;
        efldz[c] = efldz[c] - ((epres[IX(i, j, k + 1)] - epres[IX(i, j, k - 1)]) / dzt) / arho;
      }
  /* ionospheric resistance :88-116 */
  if (box <= mbndry && resist < 5000.0f) {
    const float* rst = rst_ + (size_t)(box - 1) * n;
    const int* lists[2] = {ijmid, ijzero};
    const int counts[2] = {nummid[box - 1], numzero[box - 1]};
    const int mlen[2] = {mmid, mzero};
    for (int l = 0; l < 2; l++) {
      for (int m = 1; m <= counts[l]; m++) {
        /* ij(mbndry,3,m): element (box,d,m) */
        int i = lists[l][(box - 1) + (size_t)mbndry * (0 + 3 * (size_t)(m - 1))];
        int j = lists[l][(box - 1) + (size_t)mbndry * (1 + 3 * (size_t)(m - 1))];
        int k = lists[l][(box - 1) + (size_t)mbndry * (2 + 3 * (size_t)(m - 1))];
        (void)mlen;
        const size_t c = IX(i, j, k);
        float eden = (qrho[c] / rmassq + hrho[c] / rmassh + orho[c] / rmasso);
        efldx[c] = efldx[c] + rst[c] * curx[c] / eden;
        efldy[c] = efldy[c] + rst[c] * cury[c] / eden;
        efldz[c] = efldz[c] + rst[c] * curz[c] / eden;
      }
    }
  }
  /* flank conditions :124-159 */
  const int nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;
  float* ee[3] = {efldx, efldy, efldz};
  for (int q = 0; q < 3; q++) {
    float* e = ee[q];
    for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++) {
        e[IX(1, j, k)] = e[IX(2, j, k)];
        e[IX(nx, j, k)] = e[IX(nx1, j, k)];
      }
  }
  for (int q = 0; q < 3; q++) {
    float* e = ee[q];
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        e[IX(i, j, 1)] = e[IX(i, j, 2)];
        e[IX(i, j, nz)] = e[IX(i, j, nz1)];
      }
  }
  for (int q = 0; q < 3; q++) {
    float* e = ee[q];
    for (int k = 1; k <= nz; k++)
      for (int i = 1; i <= nx; i++) {
        e[IX(i, 1, k)] = e[IX(i, 2, k)];
        e[IX(i, ny, k)] = e[IX(i, ny1, k)];
      }
  }
}

/* ======================================================================
 * lap_plasma -- sub_lap_plasma.f90:4-147; lap_elec :151-198;
 * lap_bfld :202-265.  One generic Lapidus operator, applied per field in
 * the reference's expression order.
 * ==================================================================== */
static void lapidus_field(const float* f, float* wf, float chi,
    const float* vx, const float* vy, const float* vz, float delt,
    int nx, int ny, int nz) {
  const float deltz = delt, delty = delt, deltx = delt;
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        const size_t xp = IX(i + 1, j, k), xm = IX(i - 1, j, k);
        const size_t yp = IX(i, j + 1, k), ym = IX(i, j - 1, k);
        const size_t zp = IX(i, j, k + 1), zm = IX(i, j, k - 1);
        float uxp1 = fabsf(vx[xp] - vx[c]);
        float uxm1 = fabsf(vx[c] - vx[xm]);
        float uyp1 = fabsf(vy[yp] - vy[c]);
        float uym1 = fabsf(vy[c] - vy[ym]);
        float uzp1 = fabsf(vz[zp] - vz[c]);
        float uzm1 = fabsf(vz[c] - vz[zm]);
        wf[c] = f[c] + chi * (deltx * (uxp1 * (f[xp] - f[c]) - uxm1 * (f[c] - f[xm]))
                              + delty * (uyp1 * (f[yp] - f[c]) - uym1 * (f[c] - f[ym]))
                              + deltz * (uzp1 * (f[zp] - f[c]) - uzm1 * (f[c] - f[zm])));
      }
}

void oracle_lap_plasma(const float* rho, const float* px, const float* py,
    const float* pz, const float* presx, const float* presy,
    const float* presz, const float* presxy, const float* presxz,
    const float* presyz,
    float* wrkrho, float* wrkpx, float* wrkpy, float* wrkpz,
    float* wrkpresx, float* wrkpresy, float* wrkpresz,
    float* wrkpresxy, float* wrkpresxz, float* wrkpresyz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt, int isotropic) {
  (void)n_grids; (void)chierg; (void)isotropic;
  const float* in[10] = {rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz};
  float* out[10] = {wrkrho, wrkpx, wrkpy, wrkpz, wrkpresx, wrkpresy, wrkpresz,
                    wrkpresxy, wrkpresxz, wrkpresyz};
  for (int f = 0; f < 10; f++)
    lapidus_field(BOXP(in[f]), BOXP(out[f]), f == 0 ? chirho : chipxyz,
                  vx, vy, vz, delt, nx, ny, nz);
}

void oracle_lap_elec(const float* ppres, float* wrkppres,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt) {
  (void)n_grids; (void)chirho; (void)chierg;
  lapidus_field(BOXP(ppres), BOXP(wrkppres), chipxyz, vx, vy, vz, delt, nx, ny, nz);
}

void oracle_lap_bfld(const float* bx, const float* by, const float* bz,
    float* wrkbx, float* wrkby, float* wrkbz,
    const float* vx, const float* vy, const float* vz,
    int nx, int ny, int nz, int n_grids, int box,
    float chirho, float chipxyz, float chierg, float delt) {
  (void)n_grids; (void)chirho; (void)chipxyz;
  lapidus_field(BOXP(bx), BOXP(wrkbx), chierg, vx, vy, vz, delt, nx, ny, nz);
  lapidus_field(BOXP(by), BOXP(wrkby), chierg, vx, vy, vz, delt, nx, ny, nz);
  lapidus_field(BOXP(bz), BOXP(wrkbz), chierg, vx, vy, vz, delt, nx, ny, nz);
}

/* ======================================================================
 * fcsmooth -- sub_fcsmooth.f90:7-242 (file lines 199-434 of the listing)
 * ==================================================================== */
void oracle_fcsmooth(float* px_, const float* oldpx_, const float* wrkpx_,
    int nx, int ny, int nz, int n_grids, int box, float chipx,
    float* tempx, float* tempy, float* tempz) {
  (void)n_grids; (void)tempy; (void)tempz;
  float* px = BOXP(px_);
  const float* oldpx = BOXP(oldpx_);
  const float* wrkpx = BOXP(wrkpx_);
  const size_t n = (size_t)nx * ny * nz;
  float* deltax = (float*)malloc(n * sizeof(float));
  float* delta1x = (float*)malloc(n * sizeof(float));
  float* fnx = (float*)malloc(n * sizeof(float));
  float* fny = fnx; /* the three passes never overlap in time */
  float* fnz = fnx;
  float* deltay = deltax; float* delta1y = delta1x;
  float* deltaz = deltax; float* delta1z = delta1x;

#pragma omp parallel for
  for (size_t c = 0; c < n; c++) tempx[c] = wrkpx[c];
  /* step 1: diffuse the old solution :226-243 */
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        px[c] = wrkpx[c] + chipx * (oldpx[IX(i + 1, j, k)] + oldpx[IX(i - 1, j, k)]
                                    + oldpx[IX(i, j + 1, k)] + oldpx[IX(i, j - 1, k)]
                                    + oldpx[IX(i, j, k + 1)] + oldpx[IX(i, j, k - 1)]
                                    - 6.0f * oldpx[c]);
      }
  /* boundary points :247-275 */
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      px[IX(1, j, k)] = wrkpx[IX(1, j, k)]; px[IX(nx, j, k)] = wrkpx[IX(nx, j, k)];
      tempx[IX(1, j, k)] = wrkpx[IX(1, j, k)]; tempx[IX(nx, j, k)] = wrkpx[IX(nx, j, k)];
    }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      px[IX(i, j, 1)] = wrkpx[IX(i, j, 1)]; px[IX(i, j, nz)] = wrkpx[IX(i, j, nz)];
      tempx[IX(i, j, 1)] = wrkpx[IX(i, j, 1)]; tempx[IX(i, j, nz)] = wrkpx[IX(i, j, nz)];
    }
  for (int k = 1; k <= nz; k++)
    for (int i = 1; i <= nx; i++) {
      px[IX(i, 1, k)] = wrkpx[IX(i, 1, k)]; px[IX(i, ny, k)] = wrkpx[IX(i, ny, k)];
      tempx[IX(i, 1, k)] = wrkpx[IX(i, 1, k)]; tempx[IX(i, ny, k)] = wrkpx[IX(i, ny, k)];
    }

  /* x pass :279-327 */
#pragma omp parallel for
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      for (int i = 1; i <= nx - 1; i++) {
        deltax[IX(i, j, k)] = wrkpx[IX(i + 1, j, k)] - wrkpx[IX(i, j, k)];
        delta1x[IX(i, j, k)] = px[IX(i + 1, j, k)] - px[IX(i, j, k)];
      }
      deltax[IX(nx, j, k)] = deltax[IX(nx - 1, j, k)];
      delta1x[IX(nx, j, k)] = delta1x[IX(nx - 1, j, k)];
      for (int i = 2; i <= nx - 1; i++) {
        float s = sign1(deltax[IX(i, j, k)]);
        fnx[IX(i, j, k)] = s * amax1(0.0f, amin1(amin1(s * delta1x[IX(i - 1, j, k)],
                                                       chipx * fabsf(deltax[IX(i, j, k)])),
                                                 s * delta1x[IX(i + 1, j, k)]));
      }
      fnx[IX(1, j, k)] = fnx[IX(2, j, k)];
      fnx[IX(nx, j, k)] = fnx[IX(nx - 1, j, k)];
      for (int i = 2; i <= nx - 1; i++)
        tempx[IX(i, j, k)] = px[IX(i, j, k)] - fnx[IX(i, j, k)] + fnx[IX(i - 1, j, k)];
    }

  /* y pass :331-381 */
#pragma omp parallel for
  for (int k = 1; k <= nz; k++)
    for (int i = 1; i <= nx; i++) {
      for (int j = 1; j <= ny - 1; j++) {
        deltay[IX(i, j, k)] = wrkpx[IX(i, j + 1, k)] - wrkpx[IX(i, j, k)];
        delta1y[IX(i, j, k)] = px[IX(i, j + 1, k)] - px[IX(i, j, k)];
      }
      deltay[IX(i, ny, k)] = deltay[IX(i, ny - 1, k)];
      delta1y[IX(i, ny, k)] = delta1y[IX(i, ny - 1, k)];
      for (int j = 2; j <= ny - 1; j++) {
        float s = sign1(deltay[IX(i, j, k)]);
        fny[IX(i, j, k)] = s * amax1(0.0f, amin1(amin1(s * delta1y[IX(i, j - 1, k)],
                                                       chipx * fabsf(deltay[IX(i, j, k)])),
                                                 s * delta1y[IX(i, j + 1, k)]));
      }
      fny[IX(i, 1, k)] = fny[IX(i, 2, k)];
      fny[IX(i, ny, k)] = fny[IX(i, ny - 1, k)];
      for (int j = 2; j <= ny - 1; j++)
        tempx[IX(i, j, k)] = tempx[IX(i, j, k)] - fny[IX(i, j, k)] + fny[IX(i, j - 1, k)];
    }

  /* z pass :385-431 */
#pragma omp parallel for
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      for (int k = 1; k <= nz - 1; k++) {
        deltaz[IX(i, j, k)] = wrkpx[IX(i, j, k + 1)] - wrkpx[IX(i, j, k)];
        delta1z[IX(i, j, k)] = px[IX(i, j, k + 1)] - px[IX(i, j, k)];
      }
      deltaz[IX(i, j, nz)] = deltaz[IX(i, j, nz - 1)];
      delta1z[IX(i, j, nz)] = delta1z[IX(i, j, nz - 1)];
      for (int k = 2; k <= nz - 1; k++) {
        float s = sign1(deltaz[IX(i, j, k)]);
        fnz[IX(i, j, k)] = s * amax1(0.0f, amin1(amin1(s * delta1z[IX(i, j, k - 1)],
                                                       chipx * fabsf(deltaz[IX(i, j, k)])),
                                                 s * delta1z[IX(i, j, k + 1)]));
      }
      fnz[IX(i, j, 1)] = fnz[IX(i, j, 2)];
      fnz[IX(i, j, nz)] = fnz[IX(i, j, nz - 1)];
    }
#pragma omp parallel for
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++)
        px[IX(i, j, k)] = tempx[IX(i, j, k)] - fnz[IX(i, j, k)] + fnz[IX(i, j, k - 1)];
  free(deltax); free(delta1x); free(fnx);
}

void oracle_flux_correct(float* const cur[G3M3_NFIELDS],
    float* const wrk[G3M3_NFIELDS], float* const old[G3M3_NFIELDS],
    float* vvx, float* vvy, float* vvz,
    int nx, int ny, int nz, int n_grids, int box,
    float difrho, float diferg) {
  /* the reference's call order :111-189 is per field; fields do not
   * interact, so the table order is immaterial */
  for (int f = 0; f < G3M3_NFIELDS; f++) {
    float chi = (f >= G3M3_F_BX) ? diferg : difrho;
    oracle_fcsmooth(cur[f], old[f], wrk[f], nx, ny, nz, n_grids, box, chi, vvx, vvy, vvz);
  }
}

/* ======================================================================
 * set_rho -- sub_set_rho.f90:5-104
 * ==================================================================== */
void oracle_set_rho(float* qrho_, float* qpresx_, float* qpresy_, float* qpresz_,
    float* qpresxy_, float* qpresxz_, float* qpresyz_, float rmassq,
    float* hrho_, float* hpresx_, float* hpresy_, float* hpresz_,
    float* hpresxy_, float* hpresxz_, float* hpresyz_, float rmassh,
    float* orho_, float* opresx_, float* opresy_, float* opresz_,
    float* opresxy_, float* opresxz_, float* opresyz_, float rmasso,
    float* epres_, int nx, int ny, int nz, int n_grids, int box, float o_conc) {
  (void)n_grids; (void)o_conc; (void)rmassq; (void)rmassh; (void)rmasso;
  float* rho[3] = {BOXP(qrho_), BOXP(hrho_), BOXP(orho_)};
  float* pxx[3] = {BOXP(qpresx_), BOXP(hpresx_), BOXP(opresx_)};
  float* pyy[3] = {BOXP(qpresy_), BOXP(hpresy_), BOXP(opresy_)};
  float* pzz[3] = {BOXP(qpresz_), BOXP(hpresz_), BOXP(opresz_)};
  float* pxy[3] = {BOXP(qpresxy_), BOXP(hpresxy_), BOXP(opresxy_)};
  float* pxz[3] = {BOXP(qpresxz_), BOXP(hpresxz_), BOXP(opresxz_)};
  float* pyz[3] = {BOXP(qpresyz_), BOXP(hpresyz_), BOXP(opresyz_)};
  float* epres = BOXP(epres_);
  const float mins[3] = {2.e-4f, 1.e-4f, 2.e-5f};
  const size_t n = (size_t)nx * ny * nz;
  /* (tden, rhdens, rodens of :40-44 are computed but never used) */
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    for (int s = 0; s < 3; s++) {
      if (rho[s][c] < mins[s] || pxx[s][c] < 0.0f || pyy[s][c] < 0.0f || pzz[s][c] < 0.0f) {
        rho[s][c] = amax1(fabsf(rho[s][c]), 1.05f * mins[s]);
        float apres = (fabsf(pxx[s][c]) + fabsf(pyy[s][c]) + fabsf(pzz[s][c])) / 3.0f;
        pxx[s][c] = apres; pyy[s][c] = apres; pzz[s][c] = apres;
        pxy[s][c] = 0.0f; pxz[s][c] = 0.0f; pyz[s][c] = 0.0f;
      }
    }
    epres[c] = fabsf(epres[c]);
  }
}

/* ======================================================================
 * set_speed_agrd -- sub_set_speed_agrd.f90:6-435
 * ==================================================================== */
/* iso_flag is an initialised local, hence SAVEd: once a call sees
 * isotropic=.true. it stays 0 for every later call (:68, :75). */
static float g_iso_flag = 1.0f;

void oracle_set_speed_agrd(int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, int isotropic, float smallbit,
    float aniso_limit, float vlim, float qvlim, float hvlim, float ovlim,
    float qclim, float hclim, float oclim, float cslim,
    const float* bx_, const float* by_, const float* bz_,
    const float* bx0_, const float* by0_, const float* bz0_,
    float* qrho_, float* qpx_, float* qpy_, float* qpz_,
    float* qpresx_, float* qpresy_, float* qpresz_,
    float* qpresxy_, float* qpresxz_, float* qpresyz_,
    float* hrho_, float* hpx_, float* hpy_, float* hpz_,
    float* hpresx_, float* hpresy_, float* hpresz_,
    float* hpresxy_, float* hpresxz_, float* hpresyz_,
    float* orho_, float* opx_, float* opy_, float* opz_,
    float* opresx_, float* opresy_, float* opresz_,
    float* opresxy_, float* opresxz_, float* opresyz_,
    float* epres_, float* btot,
    float* pxmax, float* pymax, float* pzmax, float* csmax, float* alfmax,
    float* fastest) {
  (void)n_grids; (void)rmassq; (void)rmassh; (void)rmasso;
  if (isotropic) g_iso_flag = 0.0f;
  const float iso_flag = g_iso_flag;
  *fastest = 0.0f; *pxmax = 0.0f; *pymax = 0.0f; *pzmax = 0.0f; *csmax = 0.0f; *alfmax = 0.0f;
  const size_t n = (size_t)nx * ny * nz;
  float* sn = (float*)malloc(13 * n * sizeof(float));
  float *srho = sn, *spx = sn + n, *spy = sn + 2 * n, *spz = sn + 3 * n;
  float *sprx = sn + 4 * n, *spry = sn + 5 * n, *sprz = sn + 6 * n;
  float *sprxy = sn + 7 * n, *sprxz = sn + 8 * n, *spryz = sn + 9 * n;
  float *bsx = sn + 10 * n, *bsy = sn + 11 * n, *bsz = sn + 12 * n;

  float* R[3] = {BOXP(qrho_), BOXP(hrho_), BOXP(orho_)};
  float* PX[3] = {BOXP(qpx_), BOXP(hpx_), BOXP(opx_)};
  float* PY[3] = {BOXP(qpy_), BOXP(hpy_), BOXP(opy_)};
  float* PZ[3] = {BOXP(qpz_), BOXP(hpz_), BOXP(opz_)};
  float* XX[3] = {BOXP(qpresx_), BOXP(hpresx_), BOXP(opresx_)};
  float* YY[3] = {BOXP(qpresy_), BOXP(hpresy_), BOXP(opresy_)};
  float* ZZ[3] = {BOXP(qpresz_), BOXP(hpresz_), BOXP(opresz_)};
  float* XY[3] = {BOXP(qpresxy_), BOXP(hpresxy_), BOXP(opresxy_)};
  float* XZ[3] = {BOXP(qpresxz_), BOXP(hpresxz_), BOXP(opresxz_)};
  float* YZ[3] = {BOXP(qpresyz_), BOXP(hpresyz_), BOXP(opresyz_)};
  const float svlim[3] = {qvlim, hvlim, ovlim};
  const float sclim[3] = {qclim, hclim, oclim};
  float mx = 0.0f, my = 0.0f, mz = 0.0f, mc = 0.0f;

  for (int s = 0; s < 3; s++) {
    float *rho = R[s], *px = PX[s], *py = PY[s], *pz = PZ[s];
    float *prx = XX[s], *pry = YY[s], *prz = ZZ[s];
    float *prxy = XY[s], *prxz = XZ[s], *pryz = YZ[s];
    /* snapshot with anisotropy limiting :88-121 */
#pragma omp parallel for
    for (size_t c = 0; c < n; c++) {
      srho[c] = rho[c]; spx[c] = px[c]; spy[c] = py[c]; spz[c] = pz[c];
      float apres = (prx[c] + pry[c] + prz[c]) / 3.0f;
      sprx[c] = aniso_limit * prx[c] + (1.0f - aniso_limit) * apres;
      spry[c] = aniso_limit * pry[c] + (1.0f - aniso_limit) * apres;
      sprz[c] = aniso_limit * prz[c] + (1.0f - aniso_limit) * apres;
      sprxy[c] = aniso_limit * prxy[c];
      sprxz[c] = aniso_limit * prxz[c];
      spryz[c] = aniso_limit * pryz[c];
    }
    if (isotropic) {
      for (size_t c = 0; c < n; c++) {
        sprx[c] = prx[c]; spry[c] = prx[c]; sprz[c] = prx[c];
        sprxy[c] = 0.0f; sprxz[c] = 0.0f; spryz[c] = 0.0f;
      }
    }
    /* limit speeds :123-184 (serial in the reference; the neighbour means
     * read only the snapshot, so the iterations are independent) */
    const float vl = vlim * svlim[s];
    const float cl = vlim * svlim[s] * sclim[s];
#pragma omp parallel for reduction(max : mx, my, mz, mc)
    for (int k = 2; k <= nz - 1; k++)
      for (int j = 2; j <= ny - 1; j++)
        for (int i = 2; i <= nx - 1; i++) {
          const size_t c = IX(i, j, k);
          const size_t xp = IX(i + 1, j, k), xm = IX(i - 1, j, k);
          const size_t yp = IX(i, j + 1, k), ym = IX(i, j - 1, k);
          const size_t zp = IX(i, j, k + 1), zm = IX(i, j, k - 1);
          float arho = rho[c] + smallbit;
          float avx = fabsf(px[c] / arho);
          float avy = fabsf(py[c] / arho);
          float avz = fabsf(pz[c] / arho);
          float vq = sqrtf(avx * avx + avy * avy + avz * avz);
          float cq = sqrtf(0.33f * (prx[c] + pry[c] + prz[c]) / arho);
          if ((vq > vl) || (cq > cl)) {
#define NMEAN(a) ((a[xp] + a[xm] + a[yp] + a[ym] + a[zp] + a[zm]) / 6.0f)
#define NMEANI(a) (iso_flag * (a[xp] + a[xm] + a[yp] + a[ym] + a[zp] + a[zm]) / 6.0f)
            rho[c] = NMEAN(srho);
            px[c] = NMEAN(spx); py[c] = NMEAN(spy); pz[c] = NMEAN(spz);
            prx[c] = NMEAN(sprx); pry[c] = NMEAN(spry); prz[c] = NMEAN(sprz);
            prxy[c] = NMEANI(sprxy); prxz[c] = NMEANI(sprxz); pryz[c] = NMEANI(spryz);
#undef NMEAN
#undef NMEANI
          }
          mx = amax1(mx, avx); my = amax1(my, avy); mz = amax1(mz, avz); mc = amax1(mc, cq);
        }
  }
  *pxmax = mx; *pymax = my; *pzmax = mz; *csmax = mc;

  /* electron pressure and Alfven speed :385-429 */
  const float *bx = BOXP(bx_), *by = BOXP(by_), *bz = BOXP(bz_);
  const float *bx0 = BOXP(bx0_), *by0 = BOXP(by0_), *bz0 = BOXP(bz0_);
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) {
    bsx[c] = bx0[c] + bx[c]; bsy[c] = by0[c] + by[c]; bsz[c] = bz0[c] + bz[c];
    btot[c] = amax1(sqrtf(bsx[c] * bsx[c] + bsy[c] * bsy[c] + bsz[c] * bsz[c]), smallbit);
  }
  float* epres = BOXP(epres_);
  float ma = 0.0f;
#pragma omp parallel for reduction(max : ma)
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        float arho = R[0][c] + R[1][c] + R[2][c] + smallbit;
        float cs = sqrtf(epres[c] / arho);
        if (cs > cslim) epres[c] = epres[c] * cslim / cs;
        ma = amax1(ma, btot[c] / sqrtf(arho));
      }
  *alfmax = ma;
  *fastest = amax1(*fastest, sqrtf(mx * mx + my * my + mz * mz + mc * mc + ma * ma));
  free(sn);
}

/* store_array -- sub_store_array.f90:1-20 (note: argument 1 is written) */
void oracle_store_array(float* bx, const float* bx0,
    int nx, int ny, int nz, int n_grids, int box) {
  (void)n_grids;
  float* d = BOXP(bx);
  const float* s = BOXP(bx0);
  memcpy(d, s, (size_t)nx * ny * nz * sizeof(float));
}

/* ======================================================================
 * flanks -- sub_flanks.f90:5-303
 * ==================================================================== */
void oracle_flanks(float* wrkrho, const float* rho, const float* oldrho,
    int nx, int ny, int nz, int n_grids, int box,
    const double* t_new, const double* t_old, double t, float* work,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax) {
  (void)n_grids;
  const int mb = box + 1, ms = box;
  const size_t n = (size_t)nx * ny * nz;
  const float t1 = (float)((t_new[mb - 1] - t) / (t_new[mb - 1] - t_old[mb - 1]));
  const float t2 = 1.0f - t1;
  const float delx = (grd_xmax[mb - 1] - grd_xmin[mb - 1]) / ((float)nx - 1.0f);
  const float dely = (grd_ymax[mb - 1] - grd_ymin[mb - 1]) / ((float)ny - 1.0f);
  const float delz = (grd_zmax[mb - 1] - grd_zmin[mb - 1]) / ((float)nz - 1.0f);
  const float sx = (grd_xmax[ms - 1] - grd_xmin[ms - 1]) / ((float)nx - 1.0f);
  const float sy = (grd_ymax[ms - 1] - grd_ymin[ms - 1]) / ((float)ny - 1.0f);
  const float sz = (grd_zmax[ms - 1] - grd_zmin[ms - 1]) / ((float)nz - 1.0f);
  const float* oc = oldrho + (size_t)(mb - 1) * n;
  const float* cc = rho + (size_t)(mb - 1) * n;
  float* w = wrkrho + (size_t)(ms - 1) * n;
  /* time interpolation of the coarse box :34-41 */
#pragma omp parallel for
  for (size_t c = 0; c < n; c++) work[c] = oc[c] * t1 + cc[c] * t2;

#define FL_COORD(axis_min_s, s_sp, idx, axis_min_b, del, ib, ib1, d, dd) \
  do {                                                                   \
    float a_ = axis_min_s + s_sp * (float)((idx) - 1);                   \
    float ai_ = 1.0f + (a_ - (axis_min_b)) / (del);                      \
    ib = (int)ai_; ib1 = ib + 1; d = ai_ - (float)ib; dd = 1.0f - d;     \
  } while (0)
#define FL_APPLY(is, js, ks, frac, frac1)                                                     \
  do {                                                                                        \
    size_t c_ = IX(is, js, ks);                                                               \
    w[c_] = frac * w[c_] + frac1 * (work[IX(ib, jb, kb)] * ddx * ddy * ddz                    \
                                    + work[IX(ib, jb, kb1)] * ddx * ddy * dz                  \
                                    + work[IX(ib, jb1, kb)] * ddx * dy * ddz                  \
                                    + work[IX(ib, jb1, kb1)] * ddx * dy * dz                  \
                                    + work[IX(ib1, jb, kb)] * dx * ddy * ddz                  \
                                    + work[IX(ib1, jb, kb1)] * dx * ddy * dz                  \
                                    + work[IX(ib1, jb1, kb)] * dx * dy * ddz                  \
                                    + work[IX(ib1, jb1, kb1)] * dx * dy * dz);                \
  } while (0)

  const float gxs = grd_xmin[ms - 1], gys = grd_ymin[ms - 1], gzs = grd_zmin[ms - 1];
  const float gxb = grd_xmin[mb - 1], gyb = grd_ymin[mb - 1], gzb = grd_zmin[mb - 1];
  /* bottom (k=2 then 1) and top (k=nz-1 then nz) panels :45-129 */
  for (int side = 0; side < 2; side++)
    for (int kk = 2; kk >= 1; kk--) {
      int ks = side == 0 ? kk : nz - kk + 1;
      int kb, kb1; float dz, ddz;
      FL_COORD(gzs, sz, ks, gzb, delz, kb, kb1, dz, ddz);
      float frac = (float)(kk - 1) / 2.0f, frac1 = 1.0f - frac;
      for (int js = 1; js <= ny; js++) {
        int jb, jb1; float dy, ddy;
        FL_COORD(gys, sy, js, gyb, dely, jb, jb1, dy, ddy);
        for (int is = 1; is <= nx; is++) {
          int ib, ib1; float dx, ddx;
          FL_COORD(gxs, sx, is, gxb, delx, ib, ib1, dx, ddx);
          FL_APPLY(is, js, ks, frac, frac1);
        }
      }
    }
  /* front (j=2,1) and back (j=ny-1,ny) panels :133-216 */
  for (int side = 0; side < 2; side++)
    for (int ks = 1; ks <= nz; ks++) {
      int kb, kb1; float dz, ddz;
      FL_COORD(gzs, sz, ks, gzb, delz, kb, kb1, dz, ddz);
      for (int jj = 2; jj >= 1; jj--) {
        int js = side == 0 ? jj : ny - jj + 1;
        int jb, jb1; float dy, ddy;
        FL_COORD(gys, sy, js, gyb, dely, jb, jb1, dy, ddy);
        float frac = (float)(jj - 1) / 2.0f, frac1 = 1.0f - frac;
        for (int is = 1; is <= nx; is++) {
          int ib, ib1; float dx, ddx;
          FL_COORD(gxs, sx, is, gxb, delx, ib, ib1, dx, ddx);
          FL_APPLY(is, js, ks, frac, frac1);
        }
      }
    }
  /* left (i=2,1) and right (i=nx-1,nx) panels :220-300 */
  for (int side = 0; side < 2; side++)
    for (int ks = 1; ks <= nz; ks++) {
      int kb, kb1; float dz, ddz;
      FL_COORD(gzs, sz, ks, gzb, delz, kb, kb1, dz, ddz);
      for (int js = 1; js <= ny; js++) {
        int jb, jb1; float dy, ddy;
        FL_COORD(gys, sy, js, gyb, dely, jb, jb1, dy, ddy);
        for (int ii = 2; ii >= 1; ii--) {
          int is = side == 0 ? ii : nx - ii + 1;
          int ib, ib1; float dx, ddx;
          FL_COORD(gxs, sx, is, gxb, delx, ib, ib1, dx, ddx);
          float frac = (float)(ii - 1) / 2.0f, frac1 = 1.0f - frac;
          FL_APPLY(is, js, ks, frac, frac1);
        }
      }
    }
#undef FL_COORD
#undef FL_APPLY
}

/* ======================================================================
 * corer -- sub_corer.f90:5-55
 * ==================================================================== */
void oracle_corer(float* rho, int nx, int ny, int nz, int n_grids, int box,
    const float* grd_xmin, const float* grd_xmax, const float* grd_ymin,
    const float* grd_ymax, const float* grd_zmin, const float* grd_zmax) {
  (void)n_grids;
  const int mb = box + 1, ms = box;
  const size_t n = (size_t)nx * ny * nz;
  const float sx = (grd_xmax[ms - 1] - grd_xmin[ms - 1]) / ((float)nx - 1.0f);
  const float dx = (grd_xmax[mb - 1] - grd_xmin[mb - 1]) / ((float)nx - 1.0f);
  const float dy = (grd_ymax[mb - 1] - grd_ymin[mb - 1]) / ((float)ny - 1.0f);
  const float dz = (grd_zmax[mb - 1] - grd_zmin[mb - 1]) / ((float)nz - 1.0f);
  const int nskip = (int)(dx / sx);
  const float ai = 1.0f + (grd_xmin[ms - 1] - grd_xmin[mb - 1]) / dx;
  const int nbx1 = (int)(ai + 0.5f);
  const float aj = 1.0f + (grd_ymin[ms - 1] - grd_ymin[mb - 1]) / dy;
  const int nby1 = (int)(aj + 0.5f);
  const float ak = 1.0f + (grd_zmin[ms - 1] - grd_zmin[mb - 1]) / dz;
  const int nbz1 = (int)(ak + 0.5f);
  float* big = rho + (size_t)(mb - 1) * n;
  const float* f = rho + (size_t)(ms - 1) * n;
#pragma omp parallel for
  for (int ks = 1 + nskip; ks <= nz - nskip; ks += nskip) {
    int kb = nbz1 + (ks - 1) / nskip;
    for (int js = 1 + nskip; js <= ny - nskip; js += nskip) {
      int jb = nby1 + (js - 1) / nskip;
      for (int is = 1 + nskip; is <= nx - nskip; is += nskip) {
        int ib = nbx1 + (is - 1) / nskip;
        big[IX(ib, jb, kb)] = (6.0f * f[IX(is, js, ks)] + f[IX(is + 1, js, ks)] + f[IX(is - 1, js, ks)]
                               + f[IX(is, js + 1, ks)] + f[IX(is, js - 1, ks)]
                               + f[IX(is, js, ks + 1)] + f[IX(is, js, ks - 1)]) / 12.0f;
      }
    }
  }
}

/* ======================================================================
 * flanks_synced -- sub_flanks_synced.f90:5-141
 * ==================================================================== */
void oracle_flanks_synced(float* rho, int nx, int ny, int nz, int n_grids,
    int box, const float* grd_xmin, const float* grd_xmax,
    const float* grd_ymin, const float* grd_ymax, const float* grd_zmin,
    const float* grd_zmax) {
  (void)n_grids;
  const int mb = box + 1, ms = box;
  const size_t n = (size_t)nx * ny * nz;
  float* fs = rho + (size_t)(ms - 1) * n;
  const float* fb = rho + (size_t)(mb - 1) * n;
  const float delx = (grd_xmax[mb - 1] - grd_xmin[mb - 1]) / ((float)nx - 1.0f);
  const float dely = (grd_ymax[mb - 1] - grd_ymin[mb - 1]) / ((float)ny - 1.0f);
  const float delz = (grd_zmax[mb - 1] - grd_zmin[mb - 1]) / ((float)nz - 1.0f);
  const float sx = (grd_xmax[ms - 1] - grd_xmin[ms - 1]) / ((float)nx - 1.0f);
  const float sy = (grd_ymax[ms - 1] - grd_ymin[ms - 1]) / ((float)ny - 1.0f);
  const float sz = (grd_zmax[ms - 1] - grd_zmin[ms - 1]) / ((float)nz - 1.0f);
  const int kb_top = (int)(1.0f + (grd_zmax[ms - 1] - grd_zmin[mb - 1]) / delz);
  const int kb_bot = (int)(1.0f + (grd_zmin[ms - 1] - grd_zmin[mb - 1]) / delz);
  const int jb_top = (int)(1.0f + (grd_ymax[ms - 1] - grd_ymin[mb - 1]) / dely);
  const int jb_bot = (int)(1.0f + (grd_ymin[ms - 1] - grd_ymin[mb - 1]) / dely);
  const int ib_top = (int)(1.0f + (grd_xmax[ms - 1] - grd_xmin[mb - 1]) / delx);
  const int ib_bot = (int)(1.0f + (grd_xmin[ms - 1] - grd_xmin[mb - 1]) / delx);
#define FS_COORD(smin, sp, idx, bmin, del, b, b1, d, dd)       \
  do {                                                        \
    float a_ = (smin) + (sp) * (float)((idx) - 1);             \
    float ai_ = 1.0f + (a_ - (bmin)) / (del);                  \
    b = (int)ai_; b1 = b + 1; d = ai_ - (float)b; dd = 1.0f - d; \
  } while (0)
  /* top and bottom :44-72 */
  for (int js = 1; js <= ny; js++) {
    int jb, jb1; float dy, ddy;
    FS_COORD(grd_ymin[ms - 1], sy, js, grd_ymin[mb - 1], dely, jb, jb1, dy, ddy);
    for (int is = 1; is <= nx; is++) {
      int ib, ib1; float dx, ddx;
      FS_COORD(grd_xmin[ms - 1], sx, is, grd_xmin[mb - 1], delx, ib, ib1, dx, ddx);
      fs[IX(is, js, nz)] = fb[IX(ib, jb, kb_top)] * ddx * ddy + fb[IX(ib, jb1, kb_top)] * ddx * dy
                           + fb[IX(ib1, jb, kb_top)] * dx * ddy + fb[IX(ib1, jb1, kb_top)] * dx * dy;
      fs[IX(is, js, 1)] = fb[IX(ib, jb, kb_bot)] * ddx * ddy + fb[IX(ib, jb1, kb_bot)] * ddx * dy
                          + fb[IX(ib1, jb, kb_bot)] * dx * ddy + fb[IX(ib1, jb1, kb_bot)] * dx * dy;
    }
  }
  /* front and back :77-105 */
  for (int ks = 1; ks <= nz; ks++) {
    int kb, kb1; float dz, ddz;
    FS_COORD(grd_zmin[ms - 1], sz, ks, grd_zmin[mb - 1], delz, kb, kb1, dz, ddz);
    for (int is = 1; is <= nx; is++) {
      int ib, ib1; float dx, ddx;
      FS_COORD(grd_xmin[ms - 1], sx, is, grd_xmin[mb - 1], delx, ib, ib1, dx, ddx);
      fs[IX(is, ny, ks)] = fb[IX(ib, jb_top, kb)] * ddx * ddz + fb[IX(ib, jb_top, kb1)] * ddx * dz
                           + fb[IX(ib1, jb_top, kb)] * dx * ddz + fb[IX(ib1, jb_top, kb1)] * dx * dz;
      fs[IX(is, 1, ks)] = fb[IX(ib, jb_bot, kb)] * ddx * ddz + fb[IX(ib, jb_bot, kb1)] * ddx * dz
                          + fb[IX(ib1, jb_bot, kb)] * dx * ddz + fb[IX(ib1, jb_bot, kb1)] * dx * dz;
    }
  }
  /* left and right :109-138 */
  for (int ks = 1; ks <= nz; ks++) {
    int kb, kb1; float dz, ddz;
    FS_COORD(grd_zmin[ms - 1], sz, ks, grd_zmin[mb - 1], delz, kb, kb1, dz, ddz);
    for (int js = 1; js <= ny; js++) {
      int jb, jb1; float dy, ddy;
      FS_COORD(grd_ymin[ms - 1], sy, js, grd_ymin[mb - 1], dely, jb, jb1, dy, ddy);
      fs[IX(nx, js, ks)] = fb[IX(ib_top, jb, kb)] * ddy * ddz + fb[IX(ib_top, jb1, kb)] * dy * ddz
                           + fb[IX(ib_top, jb, kb1)] * ddy * dz + fb[IX(ib_top, jb1, kb1)] * dy * dz;
      fs[IX(1, js, ks)] = fb[IX(ib_bot, jb, kb)] * ddy * ddz + fb[IX(ib_bot, jb1, kb)] * dy * ddz
                          + fb[IX(ib_bot, jb, kb1)] * ddy * dz + fb[IX(ib_bot, jb1, kb1)] * dy * dz;
    }
  }
#undef FS_COORD
}

/* ======================================================================
 * trilin_interp -- cft_trilin_interp.f90:10-66; findgrid -- cft_findgrid.f90
 * ==================================================================== */
void oracle_trilin_interp(const float* sxyz, const float* gridpts,
    const float* qty, float* scdata) {
  /* gridpts(3,2), qty(2,2,2) column-major */
  float x0 = gridpts[0], x1 = gridpts[3];
  float y0 = gridpts[1], y1 = gridpts[4];
  float z0 = gridpts[2], z1 = gridpts[5];
  float xd = (sxyz[0] - x0) / (x1 - x0);
  float yd = (sxyz[1] - y0) / (y1 - y0);
  float zd = (sxyz[2] - z0) / (z1 - z0);
#define Q(a, b, c) qty[((a) - 1) + 2 * (((b) - 1) + 2 * ((c) - 1))]
  float edge00 = Q(1, 1, 1) * (1.0f - xd) + Q(2, 1, 1) * xd;
  float edge01 = Q(1, 1, 2) * (1.0f - xd) + Q(2, 1, 2) * xd;
  float edge10 = Q(1, 2, 1) * (1.0f - xd) + Q(2, 2, 1) * xd;
  float edge11 = Q(1, 2, 2) * (1.0f - xd) + Q(2, 2, 2) * xd;
#undef Q
  float face0 = edge00 * (1.0f - yd) + edge10 * yd;
  float face1 = edge01 * (1.0f - yd) + edge11 * yd;
  *scdata = face0 * (1.0f - zd) + face1 * zd;
}

void oracle_findgrid(const float* xyz, int n_grids, const float* grid_minvals,
    const float* grid_maxvals, const float* xspac, int* gridpt,
    float re_equiv) {
  /* grid_minvals(3,n_grids) column-major */
  const float abit = 0.001f;
  float a[3] = {xyz[0] / re_equiv, xyz[1] / re_equiv, xyz[2] / re_equiv};
  gridpt[3] = 0;
  for (int box = 1; box <= n_grids; box++) {
    const float* mn = grid_minvals + 3 * (box - 1);
    const float* mx = grid_maxvals + 3 * (box - 1);
    if (a[0] > mn[0] && a[1] > mn[1] && a[2] > mn[2] && a[0] < mx[0] && a[1] < mx[1] && a[2] < mx[2]) {
      gridpt[3] = box;
      break;
    }
  }
  if (gridpt[3] == 0) {
    gridpt[3] = n_grids;
    const float* mn = grid_minvals + 3 * (n_grids - 1);
    const float* mx = grid_maxvals + 3 * (n_grids - 1);
    for (int d = 0; d < 3; d++) {
      a[d] = amax1(a[d], mn[d] + abit);
      a[d] = amin1(a[d], mx[d] - abit);
    }
  }
  const int b = gridpt[3];
  for (int d = 0; d < 3; d++) {
    float delta_pos = a[d] - grid_minvals[3 * (b - 1) + d];
    gridpt[d] = 1 + (int)(delta_pos / xspac[b - 1]);
  }
}

/* ======================================================================
 * flux_counter (sub_flux_counter.f90:5-158): momentum summed over the
 * walls one cell inside each face (index 2 and n-1), serially in the
 * reference's loop order, then counted as inflow or outflow by the sign of
 * the ionospheric-H+ sum.
 * ==================================================================== */
static void flux_wall(float f1[3], float f2[3], float* in[3], float* out[3],
    const float gs, const float rm[3]) {
  /* first wall: inflow when hflux1 > 0 (:48-56) */
  if (f1[1] > 0) {
    for (int s = 0; s < 3; s++) *in[s] = *in[s] + f1[s] * gs / rm[s];
  } else {
    for (int s = 0; s < 3; s++) *out[s] = *out[s] - f1[s] * gs / rm[s];
  }
  /* second wall: inflow when hflux2 < 0 (:58-66) */
  if (f2[1] < 0) {
    for (int s = 0; s < 3; s++) *in[s] = *in[s] - f2[s] * gs / rm[s];
  } else {
    for (int s = 0; s < 3; s++) *out[s] = *out[s] + f2[s] * gs / rm[s];
  }
}

void oracle_flux_counter(const float* qpx, const float* qpy, const float* qpz,
    const float* hpx, const float* hpy, const float* hpz,
    const float* opx, const float* opy, const float* opz,
    int nx, int ny, int nz, int n_grids, int box,
    float rmassq, float rmassh, float rmasso, float grid_spacing,
    float* qflux_in, float* qflux_out, float* hflux_in, float* hflux_out,
    float* oflux_in, float* oflux_out) {
  (void)n_grids;
  const size_t n3 = (size_t)nx * ny * nz, o = (size_t)(box - 1) * n3;
#define A(p, i, j, k) (p)[o + (size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1))]
  const float rm[3] = {rmassq, rmassh, rmasso};
  float* in[3] = {qflux_in, hflux_in, oflux_in};
  float* out[3] = {qflux_out, hflux_out, oflux_out};
  for (int s = 0; s < 3; s++) { *in[s] = 0.0f; *out[s] = 0.0f; }
  const float* px[3] = {qpx, hpx, opx};
  const float* py[3] = {qpy, hpy, opy};
  const float* pz[3] = {qpz, hpz, opz};
  float f1[3], f2[3];
  /* x walls, i = 2 and nx-1 (:28-46) */
  for (int s = 0; s < 3; s++) { f1[s] = 0.0f; f2[s] = 0.0f; }
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++)
      for (int s = 0; s < 3; s++) {
        f1[s] = f1[s] + A(px[s], 2, j, k);
        f2[s] = f2[s] + A(px[s], nx - 1, j, k);
      }
  flux_wall(f1, f2, in, out, grid_spacing, rm);
  /* y walls, j = 2 and ny-1 (:70-88) */
  for (int s = 0; s < 3; s++) { f1[s] = 0.0f; f2[s] = 0.0f; }
  for (int k = 1; k <= nz; k++)
    for (int i = 1; i <= nx; i++)
      for (int s = 0; s < 3; s++) {
        f1[s] = f1[s] + A(py[s], i, 2, k);
        f2[s] = f2[s] + A(py[s], i, ny - 1, k);
      }
  flux_wall(f1, f2, in, out, grid_spacing, rm);
  /* z walls, k = 2 and nz-1 (:112-130) */
  for (int s = 0; s < 3; s++) { f1[s] = 0.0f; f2[s] = 0.0f; }
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++)
      for (int s = 0; s < 3; s++) {
        f1[s] = f1[s] + A(pz[s], i, j, 2);
        f2[s] = f2[s] + A(pz[s], i, j, nz - 1);
      }
  flux_wall(f1, f2, in, out, grid_spacing, rm);
#undef A
}
