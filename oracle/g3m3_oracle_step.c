/*
 * g3m3_oracle_step.c -- TEST INFRASTRUCTURE: CPU restatement of the
 * boundary routines, the div B cleaner and the main-step schedule of the
 * G3M^3 reference (rows a13, a14, a18, a20).  Pinned bitwise to the
 * reference's own routines and main loop (see g3m3_oracle.h).
 */
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include "g3m3_oracle.h"

/* The wind-face parameters as bndry_outer reads them: the identity, except
 * in the forward-mode build (dual.h), which attaches their tangents. */
#ifndef ORACLE_WIND
#define ORACLE_WIND(k, v) (v)
#endif

#define IX(i, j, k) \
  ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (size_t)((k) - 1)))

static inline float amax1(float a, float b) { return a > b ? a : b; }
static inline float amin1(float a, float b) { return a < b ? a : b; }

/* The grid description (grd_*, xspac) as the routines take it: arrays of
 * the routines' REAL type.  In the FP32 build this is an exact copy of the
 * parameter block's arrays; the FP64 build (real8.h) widens them. */
typedef struct {
  float xmin[G3M3_MAX_GRIDS], xmax[G3M3_MAX_GRIDS], ymin[G3M3_MAX_GRIDS];
  float ymax[G3M3_MAX_GRIDS], zmin[G3M3_MAX_GRIDS], zmax[G3M3_MAX_GRIDS];
  float xspac[G3M3_MAX_GRIDS];
} grid_reals;

static grid_reals grid_of(const g3m3_params* p) {
  grid_reals g;
  for (int b = 0; b < G3M3_MAX_GRIDS; b++) {
    g.xmin[b] = p->grd_xmin[b]; g.xmax[b] = p->grd_xmax[b];
    g.ymin[b] = p->grd_ymin[b]; g.ymax[b] = p->grd_ymax[b];
    g.zmin[b] = p->grd_zmin[b]; g.zmax[b] = p->grd_zmax[b];
    g.xspac[b] = p->xspac[b];
  }
  return g;
}

/* ======================================================================
 * bndry_outer -- sub_bndry_outer.f90:5-731, applied to box n_grids.
 * The reference spells every statement out per field; the rules are the
 * same for every field apart from the momentum components (abs / -abs on
 * the faces normal to them), bx on the back-wall corner lines and epres on
 * the top back-wall line, which are kept below.
 * ==================================================================== */
void oracle_bndry_outer(float* const F[G3M3_NFIELDS],
    const float* bx0_, const float* by0_, const float* bz0_,
    const g3m3_params* p) {
  const int nx = p->nx, ny = p->ny, nz = p->nz, box = p->n_grids;
  const size_t off = (size_t)(box - 1) * nx * ny * nz;
  float* f[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) f[q] = F[q] + off;
  const float* b0[3] = {bx0_ + off, by0_ + off, bz0_ + off};
  const int nx1 = nx - 1, ny1 = ny - 1, nz1 = nz - 1;

  const float ofrac = p->rho_frac * p->o_conc;
  const float frac_h = p->rmassh / p->rmassq;
  const float frac_o = p->rmasso / p->rmassq;
  /* wind at i=1 :50-103 */
  for (int k = 1; k <= nz; k++)
    for (int j = 1; j <= ny; j++) {
      const size_t c = IX(1, j, k);
      float* q = f[0]; (void)q;
      f[0][c] = ORACLE_WIND(0, p->srho); f[1][c] = ORACLE_WIND(1, p->spx); f[2][c] = ORACLE_WIND(2, p->spy); f[3][c] = ORACLE_WIND(3, p->spz);
      f[4][c] = 0.5f * ORACLE_WIND(4, p->spress); f[5][c] = f[4][c]; f[6][c] = f[4][c];
      f[10][c] = ORACLE_WIND(0, p->srho) * p->rho_frac * frac_h;
      f[11][c] = ORACLE_WIND(1, p->spx) * p->rho_frac * frac_h;
      f[12][c] = ORACLE_WIND(2, p->spy) * p->rho_frac * frac_h;
      f[13][c] = ORACLE_WIND(3, p->spz) * p->rho_frac * frac_h;
      f[14][c] = 0.5f * ORACLE_WIND(4, p->spress) * p->rho_frac; f[15][c] = f[14][c]; f[16][c] = f[14][c];
      f[20][c] = ORACLE_WIND(0, p->srho) * ofrac * frac_o;
      f[21][c] = ORACLE_WIND(1, p->spx) * ofrac * frac_o;
      f[22][c] = ORACLE_WIND(2, p->spy) * ofrac * frac_o;
      f[23][c] = ORACLE_WIND(3, p->spz) * ofrac * frac_o;
      f[24][c] = 0.5f * ORACLE_WIND(4, p->spress) * ofrac; f[25][c] = f[24][c]; f[26][c] = f[24][c];
      f[G3M3_F_EPRES][c] = f[4][c] / p->ti_te;
      for (int s = 0; s < 3; s++)
        for (int o = 7; o <= 9; o++) f[10 * s + o][c] = 0.0f;
      f[G3M3_F_BX][c] = ORACLE_WIND(5, p->sbx_wind) - b0[0][c];
      f[G3M3_F_BY][c] = ORACLE_WIND(6, p->sby_wind) - b0[1][c];
      f[G3M3_F_BZ][c] = ORACLE_WIND(7, p->sbz_wind) - b0[2][c];
    }
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    float* a = f[q];
    const int comp = q < 30 ? q % 10 : -1; /* 1,2,3 = px,py,pz */
    /* back wall i=nx :107-154 */
    for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++) {
        float v = a[IX(nx1, j, k)];
        a[IX(nx, j, k)] = comp == 1 ? fabsf(v) : v;
      }
    /* y faces :158-252 */
    for (int k = 1; k <= nz; k++)
      for (int i = 2; i <= nx; i++) {
        float v1 = a[IX(i, 2, k)], v2 = a[IX(i, ny1, k)];
        a[IX(i, 1, k)] = comp == 2 ? -fabsf(v1) : v1;
        a[IX(i, ny, k)] = comp == 2 ? fabsf(v2) : v2;
      }
    /* z top :256-302 */
    for (int j = 1; j <= ny; j++)
      for (int i = 2; i <= nx; i++) {
        float v = a[IX(i, j, nz1)];
        a[IX(i, j, nz)] = comp == 3 ? fabsf(v) : v;
      }
    /* z bottom :306-359 */
    for (int j = 1; j <= ny; j++)
      for (int i = 2; i <= nx; i++) {
        float v = a[IX(i, j, 2)];
        a[IX(i, j, 1)] = comp == 3 ? -fabsf(v) : v;
      }
    /* corner lines at the back wall :363-472 */
    for (int k = 2; k <= nz - 1; k++) {
      if (q == G3M3_F_BX) {
        a[IX(nx, 1, k)] = a[IX(nx1, 1, k)];
        a[IX(nx, ny, k)] = a[IX(nx1, ny, k)];
      } else {
        a[IX(nx, 1, k)] = (a[IX(nx1, 1, k)] + a[IX(nx, 2, k)]) / 2.0f;
        a[IX(nx, ny, k)] = (a[IX(nx1, ny, k)] + a[IX(nx, ny1, k)]) / 2.0f;
      }
    }
    /* top and bottom lines of the back wall :473-546 */
    for (int j = 2; j <= ny - 1; j++) {
      a[IX(nx, j, 1)] = a[IX(nx, j, 2)];
      if (q != G3M3_F_EPRES) a[IX(nx, j, nz)] = a[IX(nx1, j, nz)];
    }
    /* remaining edge lines :547-728 */
    for (int i = 2; i <= nx; i++) {
      a[IX(i, 1, 1)] = a[IX(i, 1, 2)];
      a[IX(i, ny, 1)] = a[IX(i, ny, 2)];
      a[IX(i, 1, nz)] = a[IX(i, 1, nz1)];
      a[IX(i, ny, nz)] = a[IX(i, ny, nz1)];
    }
  }
}

/* ======================================================================
 * bndry_inner -- sub_bndry_inner.f90:5-268 (always box mbndry)
 * ==================================================================== */
void oracle_bndry_inner(float* const F[G3M3_NFIELDS],
    const float* parm_srf, const float* parm_mid, const float* parm_zero,
    const int* ijsrf, const int* numsrf, const int* ijmid,
    const int* nummid, const int* ijzero, const int* numzero,
    int msrf, int mmid, int mzero, const g3m3_params* p) {
  (void)msrf; (void)mmid; (void)mzero;
  const int nx = p->nx, ny = p->ny, nz = p->nz, mbndry = p->mbndry;
  const int box = mbndry;
  const size_t off = (size_t)(box - 1) * nx * ny * nz;
  float* f[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) f[q] = F[q] + off;
  const float dx = (p->grd_xmax[box - 1] - p->grd_xmin[box - 1]) / ((float)nx - 1.0f);
  const float dy = (p->grd_ymax[box - 1] - p->grd_ymin[box - 1]) / ((float)ny - 1.0f);
#define IJ(list, d, m) list[(box - 1) + (size_t)mbndry * ((d) + 3 * (size_t)((m) - 1))]
#define PARM(list, qq, m) list[(box - 1) + (size_t)mbndry * (((qq) - 1) + 7 * (size_t)((m) - 1))]
  /* ionospheric surface :44-105 */
  for (int m = 1; m <= numsrf[box - 1]; m++) {
    const int i = IJ(ijsrf, 0, m), j = IJ(ijsrf, 1, m), k = IJ(ijsrf, 2, m);
    const size_t c = IX(i, j, k);
    float ay = p->grd_ymin[box - 1] + dy * (float)(j - 1);
    float ax = p->grd_xmin[box - 1] + dx * (float)(i - 1);
    float rx = ax * p->re_equiv, ry = ay * p->re_equiv;
    float vfrac = 1.0f;
    float rvy = rx * p->v_rot * vfrac;
    float rvx = -ry * p->v_rot * vfrac;
    float rvz = 0.0f;
    float qden = amax1(PARM(parm_srf, 1, m), f[0][c]);
    float hden = amax1(PARM(parm_srf, 2, m), f[10][c]);
    float oden = amax1(PARM(parm_srf, 3, m), f[20][c]);
    f[0][c] = qden; f[10][c] = hden; f[20][c] = oden;
    for (int s = 0; s < 3; s++) {
      float pr = PARM(parm_srf, 4 + s, m);
      f[10 * s + 4][c] = pr; f[10 * s + 5][c] = pr; f[10 * s + 6][c] = pr;
    }
    f[G3M3_F_EPRES][c] = PARM(parm_srf, 7, m);
    const float den[3] = {qden, hden, oden};
    for (int s = 0; s < 3; s++) {
      f[10 * s + 1][c] = den[s] * rvx;
      f[10 * s + 2][c] = den[s] * rvy;
      f[10 * s + 3][c] = den[s] * rvz;
      f[10 * s + 7][c] = 0.0f; f[10 * s + 8][c] = 0.0f; f[10 * s + 9][c] = 0.0f;
    }
  }
  /* atmosphere :109-174 and interior :178-264 */
  for (int l = 0; l < 2; l++) {
    const int* ij = l == 0 ? ijmid : ijzero;
    const float* parm = l == 0 ? parm_mid : parm_zero;
    const int cnt = l == 0 ? nummid[box - 1] : numzero[box - 1];
    for (int m = 1; m <= cnt; m++) {
      const int i = IJ(ij, 0, m), j = IJ(ij, 1, m), k = IJ(ij, 2, m);
      const size_t c = IX(i, j, k);
      for (int s = 0; s < 3; s++) f[10 * s][c] = PARM(parm, 1 + s, m);
      for (int s = 0; s < 3; s++) {
        float pr = PARM(parm, 4 + s, m);
        f[10 * s + 4][c] = pr; f[10 * s + 5][c] = pr; f[10 * s + 6][c] = pr;
      }
      f[G3M3_F_EPRES][c] = PARM(parm, 7, m);
      float ay = p->grd_ymin[box - 1] + dy * (float)(j - 1);
      float ax = p->grd_xmin[box - 1] + dx * (float)(i - 1);
      float rx = ax * p->re_equiv, ry = ay * p->re_equiv;
      float vfrac = 1.0f;
      float rvy = rx * p->v_rot * vfrac;
      float rvx = -ry * p->v_rot * vfrac;
      float rvz = 0.0f;
      for (int s = 2; s >= 0; s--) { /* o, h, q as in the source */
        f[10 * s + 1][c] = f[10 * s][c] * rvx;
        f[10 * s + 2][c] = f[10 * s][c] * rvy;
        f[10 * s + 3][c] = f[10 * s][c] * rvz;
      }
      for (int s = 0; s < 3; s++) {
        f[10 * s + 7][c] = 0.0f; f[10 * s + 8][c] = 0.0f; f[10 * s + 9][c] = 0.0f;
      }
      if (l == 1) {
        f[G3M3_F_BX][c] = 0.0f; f[G3M3_F_BY][c] = 0.0f; f[G3M3_F_BZ][c] = 0.0f;
      }
    }
  }
#undef IJ
#undef PARM
}

/* ======================================================================
 * div B: divB_correct (sub_divB_correct.f90:25-175), sparse_solver
 * (sub_sparse_solver.f90:19-159), banded_tpose (sub_banded_tpose.f90:6-33)
 * ==================================================================== */
static void banded_tpose(int nbands, int npts, const int* pos,
    const float* bm, const float* x, float* out) {
#pragma omp parallel for
  for (int i = 1; i <= npts; i++) {
    float r = 0.0f;
    for (int band = 1; band <= nbands; band++) {
      int ii = i + pos[band - 1];
      if (ii >= 1 && ii <= npts)
        r = r + bm[(band - 1) + (size_t)nbands * (size_t)(ii - 1)] * x[ii - 1];
    }
    out[i - 1] = r;
  }
}

/* redos is initialised in its declaration, so it is SAVEd and shared by
 * every recursion level (:45). */
static int g_redos = 0;

static int sparse_solver(int nbands, int npts, const int* pos, float errlim,
    int recurse, int redo_lim, const float* divb, float* soln,
    float* residual2, float* bm) {
  float* g = (float*)malloc((size_t)npts * sizeof(float));
  float* h = (float*)malloc((size_t)npts * sizeof(float));
  float* xi = (float*)malloc((size_t)npts * sizeof(float));
  float* xj = (float*)malloc((size_t)npts * sizeof(float));
  int iters = 0;
  float errlim2 = (float)npts * (errlim * errlim);
  g_redos = recurse ? redo_lim : 0;
  g_redos = g_redos + 1;
  banded_tpose(nbands, npts, pos, bm, soln, xi);
  float divb_resd = 0.0f, sum_bsqd = 0.0f;
  for (int j = 0; j < npts; j++) {
    sum_bsqd = sum_bsqd + divb[j] * divb[j];
    xi[j] = xi[j] - divb[j];
    divb_resd = divb_resd + xi[j] * xi[j];
  }
  banded_tpose(nbands, npts, pos, bm, xi, g);
  for (int j = 0; j < npts; j++) { g[j] = -g[j]; h[j] = g[j]; }
  const long maxit = 10L * npts;
  for (long iter = 1; iter <= maxit; iter++) {
    iters = (int)iter;
    banded_tpose(nbands, npts, pos, bm, h, xi);
    float anum = 0.0f, aden = 0.0f;
    for (int j = 0; j < npts; j++) {
      anum = anum + g[j] * h[j];
      aden = aden + xi[j] * xi[j];
    }
    anum = anum / aden;
    for (int j = 0; j < npts; j++) {
      xi[j] = soln[j];
      soln[j] = soln[j] + anum * h[j];
    }
    banded_tpose(nbands, npts, pos, bm, soln, xj);
    float r2 = 0.0f;
    for (int j = 0; j < npts; j++) {
      xj[j] = xj[j] - divb[j];
      r2 = r2 + xj[j] * xj[j];
    }
    *residual2 = r2;
    if (r2 == divb_resd || r2 <= sum_bsqd * errlim2) goto done;
    if (r2 > divb_resd) {
      for (int j = 0; j < npts; j++) soln[j] = xi[j];
      if (g_redos >= 3) goto done;
      sparse_solver(nbands, npts, pos, errlim, 1, g_redos, divb, soln, residual2, bm);
    }
    divb_resd = *residual2;
    banded_tpose(nbands, npts, pos, bm, xj, xi);
    float gg = 0.0f, dgg = 0.0f;
    for (int j = 0; j < npts; j++) {
      gg = gg + g[j] * g[j];
      dgg = dgg + (xi[j] + g[j]) * xi[j];
    }
    if (gg == 0.0f) goto done;
    float gam = dgg / gg;
    for (int j = 0; j < npts; j++) {
      g[j] = -xi[j];
      h[j] = g[j] + gam * h[j];
    }
  }
done:
  free(g); free(h); free(xi); free(xj);
  return iters;
}

int oracle_sparse_solver(int nbands, int npts, const int* divb_band_pos,
    float divb_errlim, int recurse, int redo_lim, const float* divb,
    float* soln_vec, float* residual2, float* banded_matrix) {
  return sparse_solver(nbands, npts, divb_band_pos, divb_errlim, recurse, redo_lim, divb, soln_vec, residual2,
                       banded_matrix);
}

int oracle_divb_correct(int nx, int ny, int nz, int n_grids, int box,
    int nbands, const int* divb_band_pos, const float* xspac,
    float divb_errlim, float* bx_, float* by_, float* bz_) {
  (void)n_grids;
  const size_t n = (size_t)nx * ny * nz;
  const int npts = (int)n;
  float* bx = bx_ + (size_t)(box - 1) * n;
  float* by = by_ + (size_t)(box - 1) * n;
  float* bz = bz_ + (size_t)(box - 1) * n;
  const float rx = xspac[box - 1], ry = xspac[box - 1], rz = xspac[box - 1];
  float* bm = (float*)calloc((size_t)nbands * n, sizeof(float));
  float* divb = (float*)calloc(n, sizeof(float));
  float* soln = (float*)calloc(n, sizeof(float)); /* x0 = 0 (see header) */
  float* poten = (float*)calloc(n, sizeof(float));
  const int bd_low3 = 7, bd_low2 = 6, bd_low1 = 5, bd_diag = 4;
  const int bd_upp1 = 3, bd_upp2 = 2, bd_upp3 = 1;
#define BM(band, m) bm[((band) - 1) + (size_t)nbands * (size_t)((m) - 1)]
  /* banded matrix :85-123 */
  for (int m = 1; m <= npts; m++) BM(bd_diag, m) = -6.0f;
  for (int k = 1; k <= nz; k++) {
    for (int j = 1; j <= ny; j++) {
      for (int i = 2; i <= nx; i++) BM(bd_upp1, i + nx * (j - 1) + nx * ny * (k - 1)) = 1.0f;
      for (int i = 1; i <= nx - 1; i++) BM(bd_low1, i + nx * (j - 1) + nx * ny * (k - 1)) = 1.0f;
    }
    for (int j = nx + 1; j <= nx * ny; j++) BM(bd_upp2, j + nx * ny * (k - 1)) = 1.0f;
    for (int j = 1; j <= nx * ny - nx; j++) BM(bd_low2, j + nx * ny * (k - 1)) = 1.0f;
  }
  for (int j = ny * nx + 1; j <= npts; j++) BM(bd_upp3, j) = 1.0f;
  for (int j = 1; j <= npts - nx * ny; j++) BM(bd_low3, j) = 1.0f;
#undef BM
  /* divergence :130-141 */
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        divb[IX(i, j, k)] = ((bx[IX(i + 1, j, k)] - bx[IX(i - 1, j, k)])
                             + (by[IX(i, j + 1, k)] - by[IX(i, j - 1, k)])
                             + (bz[IX(i, j, k + 1)] - bz[IX(i, j, k - 1)])) / (2.0f * rx);
      }
  float residual2 = 0.0f;
  int it = sparse_solver(nbands, npts, divb_band_pos, divb_errlim, 0, 0, divb, soln, &residual2, bm);
  const float scale = rx * rx;
  for (size_t c = 0; c < n; c++) poten[c] = scale * soln[c];
  for (int k = 2; k <= nz - 1; k++)
    for (int j = 2; j <= ny - 1; j++)
      for (int i = 2; i <= nx - 1; i++) {
        const size_t c = IX(i, j, k);
        float dbx = (poten[IX(i + 1, j, k)] - poten[IX(i - 1, j, k)]) / (2.0f * rx);
        float dby = (poten[IX(i, j + 1, k)] - poten[IX(i, j - 1, k)]) / (2.0f * ry);
        float dbz = (poten[IX(i, j, k + 1)] - poten[IX(i, j, k - 1)]) / (2.0f * rz);
        bx[c] = bx[c] - dbx;
        by[c] = by[c] - dby;
        bz[c] = bz[c] - dbz;
      }
  free(bm); free(divb); free(soln); free(poten);
  return it;
}

/* ======================================================================
 * The main step -- 3d_main.f90:1925-3095
 * ==================================================================== */
static void set_rho_box(const g3m3_params* p, float* const f[G3M3_NFIELDS], int box) {
  oracle_set_rho(f[0], f[4], f[5], f[6], f[7], f[8], f[9], p->rmassq,
                 f[10], f[14], f[15], f[16], f[17], f[18], f[19], p->rmassh,
                 f[20], f[24], f[25], f[26], f[27], f[28], f[29], p->rmasso,
                 f[G3M3_F_EPRES], p->nx, p->ny, p->nz, p->n_grids, box, p->o_conc);
}

static float set_speed_box(const g3m3_params* p, oracle_state* s,
                           float* const f[G3M3_NFIELDS], int box) {
  float pxmax, pymax, pzmax, csmax, alfmax, fastest;
  const float vlim = p->vlim_factor * (float)box;
  oracle_set_speed_agrd(p->nx, p->ny, p->nz, p->n_grids, box, p->rmassq, p->rmassh,
      p->rmasso, p->isotropic, p->smallbit, p->aniso_limit, vlim, p->qvlim, p->hvlim,
      p->ovlim, p->qclim, p->hclim, p->oclim, p->cslim,
      f[G3M3_F_BX], f[G3M3_F_BY], f[G3M3_F_BZ], s->b0[0], s->b0[1], s->b0[2],
      f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9],
      f[10], f[11], f[12], f[13], f[14], f[15], f[16], f[17], f[18], f[19],
      f[20], f[21], f[22], f[23], f[24], f[25], f[26], f[27], f[28], f[29],
      f[G3M3_F_EPRES], s->btot, &pxmax, &pymax, &pzmax, &csmax, &alfmax, &fastest);
  return fastest;
}

static void bndry_corer_box(const g3m3_params* p, float* const f[G3M3_NFIELDS], int box) {
  const grid_reals g = grid_of(p);
  for (int q = 0; q < G3M3_NFIELDS; q++)
    oracle_corer(f[q], p->nx, p->ny, p->nz, p->n_grids, box, g.xmin, g.xmax,
                 g.ymin, g.ymax, g.zmin, g.zmax);
}

static void bndry_flanks_box(const g3m3_params* p, oracle_state* s,
    float* const target[G3M3_NFIELDS], float* const cur[G3M3_NFIELDS],
    float* const old[G3M3_NFIELDS], int box, double t_grid) {
  const grid_reals g = grid_of(p);
  for (int q = 0; q < G3M3_NFIELDS; q++)
    oracle_flanks(target[q], cur[q], old[q], p->nx, p->ny, p->nz, p->n_grids, box,
                  s->t_new, s->t_old, t_grid, s->vv[0], g.xmin, g.xmax,
                  g.ymin, g.ymax, g.zmin, g.zmax);
}

static void bndry_inner_all(const g3m3_params* p, oracle_state* s, float* const f[G3M3_NFIELDS]) {
  oracle_bndry_inner(f, s->parm_srf, s->parm_mid, s->parm_zero, s->ijsrf, s->numsrf,
                     s->ijmid, s->nummid, s->ijzero, s->numzero, s->msrf, s->mmid,
                     s->mzero, p);
}

static void push_ions(const g3m3_params* p, oracle_state* s, float* const out[G3M3_NFIELDS],
    float* const old[G3M3_NFIELDS], float* const src[G3M3_NFIELDS], int box, float delt) {
  const grid_reals g = grid_of(p);
  const float masses[3] = {p->rmassq, p->rmassh, p->rmasso};
  for (int sp = 0; sp < 3; sp++) {
    const int b = 10 * sp;
    oracle_push_ion(out[b + 0], out[b + 4], out[b + 5], out[b + 6], out[b + 1], out[b + 2], out[b + 3],
                    old[b + 0], old[b + 4], old[b + 5], old[b + 6], old[b + 1], old[b + 2], old[b + 3],
                    src[b + 0], src[b + 4], src[b + 5], src[b + 6], src[b + 1], src[b + 2], src[b + 3],
                    out[b + 7], out[b + 8], out[b + 9], old[b + 7], old[b + 8], old[b + 9],
                    src[b + 7], src[b + 8], src[b + 9],
                    s->bs[0], s->bs[1], s->bs[2], s->btot, s->efld[0], s->efld[1], s->efld[2],
                    masses[sp], s->vv[0], s->vv[1], s->vv[2], s->tv[0], s->tv[1], s->tv[2],
                    p->gamma, p->gamma1, p->nx, p->ny, p->nz, p->n_grids, box, delt, p->grav,
                    p->re_equiv, p->reynolds, g.xmin, g.xmax, g.ymin,
                    g.ymax, g.zmin, g.zmax, p->isotropic);
  }
}

/* calcur, bs/btot, fnd_evel and BandE for the state f of one box */
static void fields_for(const g3m3_params* p, oracle_state* s, float* const f[G3M3_NFIELDS],
                       int box, float rx) {
  const int nx = p->nx, ny = p->ny, nz = p->nz, ng = p->n_grids;
  oracle_calcur(f[G3M3_F_BX], f[G3M3_F_BY], f[G3M3_F_BZ], nx, ny, nz, ng, box,
                s->curr[0], s->curr[1], s->curr[2], rx, rx, rx);
  oracle_total_b(f[G3M3_F_BX], f[G3M3_F_BY], f[G3M3_F_BZ], s->b0[0], s->b0[1], s->b0[2],
                 nx, ny, nz, ng, box, p->smallbit, s->bs[0], s->bs[1], s->bs[2], s->btot);
  oracle_fnd_evel(f[1], f[2], f[3], f[0], f[11], f[12], f[13], f[10], f[21], f[22], f[23], f[20],
                  s->curr[0], s->curr[1], s->curr[2], s->ev[0], s->ev[1], s->ev[2],
                  s->tv[0], s->tv[1], s->tv[2], nx, ny, nz, ng, box,
                  p->rmassq, p->rmassh, p->rmasso, p->reynolds);
  oracle_bande(s->efld[0], s->efld[1], s->efld[2], s->bs[0], s->bs[1], s->bs[2],
               s->curr[0], s->curr[1], s->curr[2], s->ev[0], s->ev[1], s->ev[2], s->btot,
               f[G3M3_F_EPRES], f[0], f[10], f[20], s->resistive, p->resist, p->reynolds,
               nx, ny, nz, ng, box, p->rmassq, p->rmassh, p->rmasso,
               s->ijmid, s->nummid, s->ijzero, p->mbndry, s->numzero, s->mmid, s->mzero,
               rx, rx, rx);
}

void oracle_init_steps(const g3m3_params* p, oracle_state* s) {
  for (int box = p->n_grids; box >= 1; box--) {
    s->t_old[box - 1] = 0.0;
    s->t_new[box - 1] = 0.0;
    set_rho_box(p, s->cur, box);
    float fastest = set_speed_box(p, s, s->cur, box);
    s->t_stepnew[box - 1] = (double)amin1(p->stepsz * p->xspac[box - 1] / fastest, p->t_step_max);
  }
}

static void box_step(const g3m3_params* p, oracle_state* s, int box) {
  const int nx = p->nx, ny = p->ny, nz = p->nz, ng = p->n_grids;
  float* const* cur = s->cur;
  float* const* old = s->old;
  float* const* wrk = s->wrk;
  s->t_old[box - 1] = s->t_new[box - 1];
  s->t_new[box - 1] = s->t_old[box - 1] + s->t_step[box - 1];
  const float delt = (float)s->t_step[box - 1];
  const float delt2 = delt / 2.0f;
  double t_grid = 0.0;
  float rx = p->xspac[box - 1];

  /* store initial values :2193-2229 */
  for (int q = 0; q < G3M3_NFIELDS; q++) oracle_store_array(old[q], cur[q], nx, ny, nz, ng, box);

  /* ---- predictor :2238-2449 ---- */
  fields_for(p, s, cur, box, rx);
  oracle_push_elec(wrk[G3M3_F_EPRES], old[G3M3_F_EPRES], cur[G3M3_F_EPRES],
                   s->ev[0], s->ev[1], s->ev[2], p->gamma, p->gamma1, nx, ny, nz, ng, box,
                   0.5f * delt, rx, rx, rx);
  push_ions(p, s, wrk, old, cur, box, 0.5f * delt);
  oracle_push_bfld(wrk[G3M3_F_BX], wrk[G3M3_F_BY], wrk[G3M3_F_BZ],
                   old[G3M3_F_BX], old[G3M3_F_BY], old[G3M3_F_BZ],
                   s->efld[0], s->efld[1], s->efld[2], nx, ny, nz, ng, box, 0.5f * delt, rx, rx, rx);
  if (box == ng) {
    oracle_bndry_outer(wrk, s->b0[0], s->b0[1], s->b0[2], p);
  } else {
    t_grid = s->t_old[box - 1] + (double)delt2;
    if (t_grid > s->t_new[box]) t_grid = s->t_new[box];
    if (t_grid < s->t_old[box]) t_grid = s->t_old[box];
    bndry_flanks_box(p, s, wrk, cur, old, box, t_grid);
  }
  if (box <= p->mbndry) bndry_inner_all(p, s, wrk);
  set_rho_box(p, wrk, box);
  (void)set_speed_box(p, s, wrk, box);

  /* ---- corrector :2481-2684 ---- */
  fields_for(p, s, wrk, box, rx);
  oracle_push_elec(wrk[G3M3_F_EPRES], old[G3M3_F_EPRES], cur[G3M3_F_EPRES],
                   s->ev[0], s->ev[1], s->ev[2], p->gamma, p->gamma1, nx, ny, nz, ng, box,
                   delt, rx, rx, rx);
  push_ions(p, s, cur, old, wrk, box, delt);
  oracle_push_bfld(cur[G3M3_F_BX], cur[G3M3_F_BY], cur[G3M3_F_BZ],
                   old[G3M3_F_BX], old[G3M3_F_BY], old[G3M3_F_BZ],
                   s->efld[0], s->efld[1], s->efld[2], nx, ny, nz, ng, box, delt, rx, rx, rx);
  if (box == ng) {
    oracle_bndry_outer(cur, s->b0[0], s->b0[1], s->b0[2], p);
  } else {
    t_grid = s->t_old[box - 1] + (double)delt;
    if (t_grid > s->t_new[box]) t_grid = s->t_new[box];
    if (t_grid < s->t_old[box]) t_grid = s->t_old[box];
    /* the reference applies these flanks to the wrk arrays (:2599-2637) */
    bndry_flanks_box(p, s, wrk, cur, old, box, t_grid);
  }
  if (box <= p->mbndry) bndry_inner_all(p, s, cur);
  set_rho_box(p, cur, box);
  (void)set_speed_box(p, s, cur, box);

  /* ---- Lapidus :2690-2887 ---- */
  for (int sp = 0; sp < 3; sp++) {
    const int b = 10 * sp;
    const size_t n = (size_t)nx * ny * nz, o = (size_t)(box - 1) * n;
    for (size_t c = 0; c < n; c++) {
      float r = amax1(cur[b][o + c], p->smallbit);
      s->curr[0][c] = cur[b + 1][o + c] / r;
      s->curr[1][c] = cur[b + 2][o + c] / r;
      s->curr[2][c] = cur[b + 3][o + c] / r;
    }
    oracle_lap_plasma(cur[b], cur[b + 1], cur[b + 2], cur[b + 3], cur[b + 4], cur[b + 5], cur[b + 6],
                      cur[b + 7], cur[b + 8], cur[b + 9],
                      wrk[b], wrk[b + 1], wrk[b + 2], wrk[b + 3], wrk[b + 4], wrk[b + 5], wrk[b + 6],
                      wrk[b + 7], wrk[b + 8], wrk[b + 9], s->curr[0], s->curr[1], s->curr[2],
                      nx, ny, nz, ng, box, p->chirho, p->chipxyz, p->chierg, delt, p->isotropic);
  }
  oracle_fnd_vtot(cur[1], cur[2], cur[3], cur[0], cur[11], cur[12], cur[13], cur[10],
                  cur[21], cur[22], cur[23], cur[20], s->curr[0], s->curr[1], s->curr[2],
                  nx, ny, nz, ng, box, p->rmassq, p->rmassh, p->rmasso);
  oracle_lap_elec(cur[G3M3_F_EPRES], wrk[G3M3_F_EPRES], s->curr[0], s->curr[1], s->curr[2],
                  nx, ny, nz, ng, box, p->chirho, p->chipxyz, p->chierg, delt);
  oracle_lap_bfld(cur[G3M3_F_BX], cur[G3M3_F_BY], cur[G3M3_F_BZ],
                  wrk[G3M3_F_BX], wrk[G3M3_F_BY], wrk[G3M3_F_BZ],
                  s->curr[0], s->curr[1], s->curr[2], nx, ny, nz, ng, box,
                  p->chirho, p->chipxyz, p->chierg, delt);
  if (box == ng) {
    oracle_bndry_outer(wrk, s->b0[0], s->b0[1], s->b0[2], p);
  } else {
    bndry_flanks_box(p, s, wrk, cur, old, box, t_grid);
  }
  if (box <= p->mbndry) bndry_inner_all(p, s, wrk);
  set_rho_box(p, wrk, box);
  (void)set_speed_box(p, s, wrk, box);

  /* ---- flux correction :2896-3039 ---- */
  oracle_flux_correct(cur, wrk, old, s->vv[0], s->vv[1], s->vv[2], nx, ny, nz, ng, box,
                      p->difrho, p->diferg);
  if (box == ng) {
    oracle_bndry_outer(cur, s->b0[0], s->b0[1], s->b0[2], p);
  } else {
    bndry_flanks_box(p, s, cur, cur, old, box, t_grid);
  }
  if (box <= p->mbndry) bndry_inner_all(p, s, cur);
  set_rho_box(p, cur, box);
  float fastest = set_speed_box(p, s, cur, box);
  s->t_stepnew[box - 1] = (double)amin1(p->stepsz * p->xspac[box - 1] / fastest, p->t_step_max);

  /* core sync :3044-3063 */
  if (box < ng) {
    if (fabs(s->t_new[box - 1] - s->t_new[box]) <= (double)0.005f * s->t_step[box - 1]) {
      bndry_corer_box(p, s->cur, box);
      s->t_old[box] = s->t_new[box];
    }
  }
  s->cell_updates += (int64_t)nx * ny * nz;
}

int oracle_main_step(const g3m3_params* p, oracle_state* s) {
  const int ng = p->n_grids;
  double smallest_step = 0.0;
  int m_smallest = ng;
  /* schedule :1929-1968 */
  for (int box = ng; box >= 1; box--) {
    s->t_step[box - 1] = s->t_stepnew[box - 1];
    s->t_old[box - 1] = 0.0;
    s->t_new[box - 1] = 0.0;
    if (box == ng) {
      smallest_step = s->t_step[box - 1];
      m_smallest = box;
    } else {
      if (s->t_step[box - 1] > s->t_step[box]) s->t_step[box - 1] = s->t_step[box];
      if (smallest_step > s->t_step[box - 1]) {
        smallest_step = s->t_step[box - 1];
        m_smallest = box;
      }
    }
  }
  for (int box = 1; box <= ng; box++) {
    if (box <= m_smallest) {
      s->t_step[box - 1] = smallest_step;
    } else {
      float astep = (float)(s->t_step[box - 1] / s->t_step[box - 2] + 0.50);
      int nsteps = (int)astep;
      if (nsteps > 2) nsteps = 2;
      if (nsteps < 1) nsteps = 1;
      s->t_step[box - 1] = s->t_step[box - 2] * nsteps;
    }
  }
  const int m_step = (int)(s->t_step[ng - 1] / s->t_step[m_smallest - 1]);
  const float delt = (float)s->t_step[ng - 1];
  if (delt < p->t_step_min) return 1;
  s->t = s->t + (double)delt;

  /* sub-cycle loop :2142-3066 */
  for (int ms = 1; ms <= m_step; ms++) {
    for (int box = ng; box >= 1; box--) {
      int yes_step = 0;
      if (box == 1) {
        yes_step = 1;
      } else if (s->t_old[box - 1] == s->t_new[box - 1] &&
                 s->t_new[box - 1] < s->t_step[ng - 1] &&
                 fabs(s->t_new[box - 1] - s->t_new[0]) <= (double)0.005f * s->t_step[0]) {
        yes_step = 1;
      }
      if (yes_step) box_step(p, s, box);
    }
  }
  /* final sync :3069-3095 */
  s->t_old[0] = s->t_new[0];
  for (int box = 1; box <= ng - 1; box++) {
    bndry_corer_box(p, s->cur, box);
    set_rho_box(p, s->cur, box);
    if (box > 1) { /* the reference reads t_old(0) for box 1 */
      s->t_old[box - 1] = s->t_old[box - 2];
      s->t_new[box - 1] = s->t_new[box - 2];
    }
  }
  s->nsteps_done += 1;
  if (p->divb_every > 0 && (s->nsteps_done % p->divb_every) == 0) oracle_divb_all(p, s);
  return 0;
}

void oracle_divb_all(const g3m3_params* p, oracle_state* s) {
  const grid_reals g = grid_of(p);
  const int nx = p->nx, ny = p->ny, ng = p->n_grids;
  const int pos[7] = {nx * ny, nx, 1, 0, -1, -nx, -nx * ny};
  for (int box = ng; box >= 1; box--) {
    for (int rep = 0; rep < 2; rep++)
      s->last_cg_iters = oracle_divb_correct(nx, ny, p->nz, ng, box, 7, pos, g.xspac,
          p->divb_errlim, s->cur[G3M3_F_BX], s->cur[G3M3_F_BY], s->cur[G3M3_F_BZ]);
  }
  for (int box = ng - 1; box >= 1; box--)
    for (int q = G3M3_F_BX; q <= G3M3_F_BZ; q++)
      oracle_flanks_synced(s->cur[q], nx, ny, p->nz, ng, box, g.xmin, g.xmax,
                           g.ymin, g.ymax, g.zmin, g.zmax);
  for (int box = 1; box <= ng - 1; box++) bndry_corer_box(p, s->cur, box);
}
