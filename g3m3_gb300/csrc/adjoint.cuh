// adjoint.cuh -- argument blocks and launchers of the reverse-mode kernels
// (k_adj.cu) that adjoint.cu runs backwards through the recorded main steps.
//
// Conventions.  For every forward array there is an adjoint array of the
// same shape ("a_" prefix).  A reverse kernel reads the adjoint of what its
// forward kernel wrote and adds J^T of it into the adjoints of what the
// forward kernel read: by atomic additions where several cells read one
// input, or as a gather, each input's thread summing the shares it receives
// (the Lapidus and flux-correction reverses).  The adjoint of every value
// the forward kernel overwrote is cleared, by the kernel or, after a
// gather that others still read, by its caller.  Primal values come from
// the tape's snapshots or are recomputed from them.
#pragma once

#include "bndry.cuh"
#include "kargs.cuh"

namespace g3m3 {

struct AdjPushIonArgs {          // push_ion (one species)
  const float* src[10];
  const float* old[10];
  const float* bs[3];
  const float* btot;
  const float* efld[3];
  const float* tv[3];
  float* a_out[10];              // read, then cleared where the push wrote
  float* a_src[10];
  float* a_old[10];
  float* a_bs[3];
  float* a_btot;
  float* a_efld[3];
  float* a_tv[3];
  Dims d;
  Geom g;
  float rmass, grav, re_equiv, reynolds, delt;
  int boundary_from_old;         // the push also wrote out = old on the boundary
};

struct AdjPushFieldArgs {        // push_elec (do_elec) and push_bfld (do_bfld)
  const float* wrkepres;
  const float* ev[3];
  float* a_epres;
  float* a_wrkepres;
  float* a_oldepres;
  float* a_ev[3];
  float* a_b[3];
  float* a_oldb[3];
  float* a_efld[3];
  Dims d;
  float rx, ry, rz, gamma, gamma1, delt;
  int do_elec, do_bfld, boundary_from_old;
};

struct AdjFieldsArgs {           // calcur + bs/btot + fnd_evel + BandE of one state
  const float* b[3];
  const float* b0[3];
  const float* rho[3];
  const float* p[3][3];
  const float* epres;
  const float* rst_e;            // BandE's resistive coefficient, or null
  const float* cur[3];           // primal scratch, recomputed from the state
  const float* bs[3];
  const float* ev[3];
  float* a_efld[3];              // adjoints of the scratch (read and cleared)
  float* a_cur[3];
  float* a_bs[3];
  float* a_btot;
  float* a_ev[3];
  float* a_tv[3];
  float* a_b[3];                 // adjoints of the state (accumulated)
  float* a_rho[3];
  float* a_p[3][3];
  float* a_epres;
  Dims d;
  float rmass[3], reynolds, rx, ry, rz, smallbit;
};

struct AdjLapArgs {              // one Lapidus call (up to 10 fields, one velocity)
  const float* in[10];
  const float* vp[3];            // v = p / max(rho, vfloor) from (vp, vrho), or explicit v
  const float* vrho;
  const float* v[3];
  float* a_out[10];
  float* a_in[10];
  float* a_vp[3];
  float* a_vrho;
  float* a_v[3];
  float chi[10];
  int nf;
  float vfloor, delt;
  Dims d;
};

struct AdjVtotArgs {             // fnd_vtot
  const float* p[3][3];
  const float* rho[3];
  float* a_v[3];
  float* a_p[3][3];
  float* a_rho[3];
  Dims d;
};

struct AdjFcsArgs {              // flux correction of nf fields
  const float* wrk[G3M3_NFIELDS];
  const float* old[G3M3_NFIELDS];
  float* p1;                     // scratch [nf][cells]: P1 = wrk + chi Lap7(old)
  float* a_p1;                   // scratch [nf][cells]: P1's adjoint (written by the gather)
  float* fm;                     // scratch [3][nf][cells]: per face and axis, the value its limiter
  float* fw;                     //   passes to d1m, dw or d1p (zero for the other two)
  float* fp;
  float* a_px[G3M3_NFIELDS];
  float* a_wrk[G3M3_NFIELDS];
  float* a_old[G3M3_NFIELDS];
  float chi[G3M3_NFIELDS];
  int nf;
  int clear_px;                  // set by the launcher: k_adj_p1 clears a_px
  Dims d;
};

struct AdjGuardArgs {            // set_rho (+ set_speed_agrd) in place
  const float* pre[G3M3_NFIELDS];   // the state before the guards
  float* a[G3M3_NFIELDS];
  Dims d;
  float smallbit, aniso_limit, vlim;
  float svlim[3], sclim[3];
  float cslim, iso_flag;
  int isotropic, do_speed;
  float* list;                   // replaced (cell, species): 1 + 10 words each
  unsigned* list_count;
  unsigned list_cap;
};

struct AdjOuterArgs {            // bndry_outer
  const float* post[G3M3_NFIELDS];  // the state after the boundary (interior unchanged)
  float* a[G3M3_NFIELDS];
  const float* b0[3];
  double* a_param;               // [8]: srho spx spy spz spress sbx sby sbz
  Dims d;
  float rmassq, rmassh, rmasso;
  float srho, rho_frac, o_conc, spress, spx, spy, spz;
  float sbx_wind, sby_wind, sbz_wind, ti_te;
};

struct AdjInnerArgs {            // bndry_inner on box mbndry
  const float* post[G3M3_NFIELDS];
  float* a[G3M3_NFIELDS];
  const int* ij[3];
  const float* parm[3];
  int num[3];
  int mbndry, box;
  Dims d;
  float xmin, ymin, dx, dy, re_equiv, v_rot;
};

struct AdjFlanksArgs {           // flanks (the fine shell from the coarse box)
  float* a_target[G3M3_NFIELDS];
  float* a_curc[G3M3_NFIELDS];
  float* a_oldc[G3M3_NFIELDS];
  int nf;
  Dims d;
  float t1;
  float sxmin, symin, szmin, sx, sy, sz;
  float bxmin, bymin, bzmin, delx, dely, delz;
};

struct AdjCorerArgs {            // corer
  float* a_coarse[G3M3_NFIELDS];
  float* a_fine[G3M3_NFIELDS];
  int nf;
  Dims d;
  int nskip, nbx1, nby1, nbz1;
  int ni, nj, nk;
};

struct AdjSyncedArgs {           // flanks_synced
  float* a_fine[G3M3_NFIELDS];
  float* a_coarse[G3M3_NFIELDS];
  int nf;
  Dims d;
  float sxmin, symin, szmin, sx, sy, sz;
  float bxmin, bymin, bzmin, delx, dely, delz;
  int kb_top, kb_bot, jb_top, jb_bot, ib_top, ib_bot;
};

struct AdjDivbArgs {             // the div B projection of one box
  float* a_b[3];                 // adjoint of B after the projection; becomes the adjoint before it
  float* rhs;                    // scratch: right-hand side and solution of the adjoint solve
  const float* z;                // the solve's solution (for the second kernel)
  Dims d;
  float rx;
};

struct LossArgs {                // virtual-spacecraft misfit of one main step
  const float* f[G3M3_MAX_GRIDS][4];   // bx, by, bz and the three densities summed on the fly
  const float* rho[G3M3_MAX_GRIDS][3];
  float* a_f[G3M3_MAX_GRIDS][3];
  float* a_rho[G3M3_MAX_GRIDS][3];
  const float* xyz;              // [n][3] positions, planet radii
  const float* target;           // [n][4]: bx by bz rho
  float* resid;                  // [n][4] value - target (forward), read by the reverse
  double* loss;
  int n, n_grids;
  Dims d;
  float gmin[3 * G3M3_MAX_GRIDS], gmax[3 * G3M3_MAX_GRIDS], xspac[G3M3_MAX_GRIDS], re_equiv;
};

void launch_adj_push_ion(const AdjPushIonArgs& a, cudaStream_t s);
void launch_adj_push_field(const AdjPushFieldArgs& a, cudaStream_t s);
void launch_adj_fields(const AdjFieldsArgs& a, cudaStream_t s);
void launch_adj_lap(const AdjLapArgs& a, cudaStream_t s);
void launch_adj_vtot(const AdjVtotArgs& a, cudaStream_t s);
void launch_adj_fcs(const AdjFcsArgs& a, cudaStream_t s);
void launch_adj_guard(const AdjGuardArgs& a, cudaStream_t s);
void launch_adj_outer(const AdjOuterArgs& a, cudaStream_t s);
void launch_adj_inner(const AdjInnerArgs& a, cudaStream_t s);
void launch_adj_flanks(const AdjFlanksArgs& a, cudaStream_t s);
void launch_adj_corer(const AdjCorerArgs& a, cudaStream_t s);
void launch_adj_synced(const AdjSyncedArgs& a, cudaStream_t s);
// div B: rhs = s G^T a_b (interior), then (after the solve of A z = rhs)
// a_b -= D^T z
void launch_adj_divb_rhs(const AdjDivbArgs& a, cudaStream_t s);
void launch_adj_divb_apply(const AdjDivbArgs& a, cudaStream_t s);
void launch_loss(const LossArgs& a, cudaStream_t s, bool reverse);
void launch_copy_fields(float* dst, const float* const src[], int nf, size_t n, cudaStream_t s);
void launch_copy_fields_out(float* const dst[], const float* src, int nf, size_t n, cudaStream_t s);
void launch_move_fields(float* dst, float* const src[], int nf, size_t n, cudaStream_t s);   // src cleared
void launch_zero(float* p, size_t n, cudaStream_t s);
void launch_axpy(float* y, const float* x, size_t n, cudaStream_t s);   // y += x

}  // namespace g3m3
