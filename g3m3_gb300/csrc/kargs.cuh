// kargs.cuh -- argument blocks of the G3M^3 kernels.
//
// Every kernel takes one of these structs by value (__grid_constant__), so a
// launch captured in a CUDA graph carries its own copy.  Pointers are box
// slices A(:,:,:,box) of the reference's (nx,ny,nz,n_grids) arrays, or
// per-box scratch A(nx,ny,nz).  Field tables use the order of g3m3_types.h:
// rho, px, py, pz, presx, presy, presz, presxy, presxz, presyz.
#pragma once

#include "common.cuh"

namespace g3m3 {

struct Geom {            // one box: origin and spacing (grd_*min, dx/dy/dz)
  float xmin, ymin, zmin;
  float dx, dy, dz;
};

struct PushIonArgs {
  float* out[10];
  const float* old[10];
  const float* src[10];
  const float* bs[3];
  const float* btot;
  const float* efld[3];
  const float* tv[3];
  Dims d;
  Geom g;
  float rmass, grav, re_equiv, reynolds;
  ScalarRef delt;
  int boundary_from_old;   // also set out = old on the boundary cells
  int contracted;          // run the contracted flavour (g3m3::contracted)
};

struct PushFieldArgs {     // push_elec and push_bfld in one pass
  const float* wrkepres;   // source of the electron pressure flux (arg 1)
  const float* oldepres;
  float* epres;            // written (arg 3)
  const float* ev[3];
  float* b[3];
  const float* oldb[3];
  const float* efld[3];
  Dims d;
  float rx, ry, rz, gamma, gamma1;
  ScalarRef delt;
  int do_elec, do_bfld;
  int boundary_from_old;
};

struct CurrentArgs {       // calcur + (optionally) bs = b0 + b, btot
  const float* b[3];
  const float* b0[3];      // null: skip bs/btot
  float* cur[3];
  float* bs[3];
  float* btot;
  Dims d;
  float rx, ry, rz, smallbit;
};

struct EvelArgs {          // fnd_evel (ev may be null: fnd_vtot)
  const float* p[3][3];    // [species][component]
  const float* rho[3];
  const float* cur[3];
  float* ev[3];
  float* tv[3];
  Dims d;
  float rmass[3], reynolds;
};

struct BandEArgs {
  float* efld[3];
  const float* bs[3];
  const float* cur[3];
  const float* ev[3];
  const float* epres;
  const float* rho[3];
  const float* rst_e;      // resistive coefficient where BandE applies it, or null
  Dims d;
  float rmass[3], reynolds, rx, ry, rz;
};

struct BandEListArgs {     // the ijmid/ijzero resistive scatter
  float* efld[3];
  const float* cur[3];
  const float* rho[3];
  const float* rst;
  const int* ij;           // (mbndry,3,m) column-major
  int count, mbndry, box;
  Dims d;
  float rmass[3];
  int serial;              // the list names a cell twice: one thread, in order
};

struct LapArgs {           // Lapidus smoothing of up to 10 fields with one velocity
  const float* in[10];
  float* out[10];
  float chi[10];
  int nf;
  // velocity: either v = p/max(rho,vfloor) from (vp, vrho) or explicit v
  const float* vp[3];
  const float* vrho;
  const float* v[3];
  float vfloor;
  Dims d;
  ScalarRef delt;
};

struct VtotArgs {          // fnd_vtot velocity written for lap_elec/lap_bfld
  const float* p[3][3];
  const float* rho[3];
  float* v[3];
  Dims d;
};

struct FcsArgs {           // fcsmooth for up to 34 fields
  float* px[G3M3_NFIELDS];
  const float* old[G3M3_NFIELDS];
  const float* wrk[G3M3_NFIELDS];
  float chi[G3M3_NFIELDS];
  int nf;
  Dims d;
  int variant;              // tile shape (launch_fcsmooth); 0 = default
};

struct GuardArgs {         // set_rho and/or set_speed_agrd
  float* f[G3M3_NFIELDS];  // 30 species fields + epres + b (b read only)
  const float* b0[3];
  float* btot;
  Dims d;
  float smallbit, aniso_limit, vlim;
  float svlim[3], sclim[3];
  float cslim, iso_flag;
  int isotropic;
  int do_set_rho, do_speed;
  // deferred replacement list (scratch): entries of 1 + 10 words
  float* list;
  unsigned int* list_count;
  unsigned int list_cap;
  unsigned int* maxbits;   // 5 words: pxmax pymax pzmax csmax alfmax (float bits)
  // The reference's running maximum restarts after a NaN; the drop-in
  // reproduces that through these words (null: plain maxima): [0] bit w set
  // when word w met a NaN, [1+w] the last NaN's position in the
  // reference's loop order + 1, [6+w] the maximum after it (float bits),
  // [11] bit w set when an element follows it.
  unsigned int* fold;
};

struct ScatterArgs {
  float* f[G3M3_NFIELDS];
  const float* list;
  const unsigned int* list_count;
  unsigned int list_cap;
};

struct FluxArgs {           // flux_counter
  const float* p[3][3];    // species (q, h, o) x momentum component (x, y, z), box slices
  Dims d;
  float rmass[3];
  float grid_spacing;
  float* out;              // 6 values (q in/out, h in/out, o in/out), or the history
  unsigned int* count;     // history mode: slot counter of the main step (null: write out[0..5])
  unsigned int capacity;   // history slots (main steps)
  int n_grids, box, advance;   // advance: this launch moves the counter on
};

struct CutArgs {            // one grid plane of up to 16 box arrays
  const float* src[16];
  int nq, q0;              // arrays, and the first output slot they fill
  int plane, index;        // 0: k = index (x-y), 1: j = index (x-z), 2: i = index (y-z)
  Dims d;
  float* out;              // [slot][a][b]
};

struct SampleArgs {
  const float* field;      // A(nx,ny,nz,n_grids)
  const float* xyz;        // (3,n)
  float* out;
  int n, n_grids;
  Dims d;
  float gmin[3 * G3M3_MAX_GRIDS], gmax[3 * G3M3_MAX_GRIDS], xspac[G3M3_MAX_GRIDS];
  float re_equiv;
};

struct InitArgs {           // fresh-start state of one box (k_init.cu)
  float* f[G3M3_NFIELDS];
  float* b0[3];
  Dims d;
  int box;
  float xmin, ymin, zmin;
  double dx, dy, dz;
  double b0c, zero_b, re_equiv, r_rot, v_rot, r_inner, alpha_e, erho, d_min, cs_inner, ti_te, gamma;
  double spress, srho, spx, spy, spz, rho_frac, rmass[3];
  float noise;
  unsigned long long seed;
};

struct CraftArgs {          // per-step virtual-spacecraft recording
  SampleArgs geo;           // grid description (field, xyz, out, n unused)
  const float* traj;        // (4, samples): x, y, z in planet radii, t
  const int* start;         // first sample of each craft, ncraft + 1 entries
  int ncraft, nf;
  const float* fld[8][G3M3_MAX_GRIDS];   // box slices of the recorded fields
  ScalarRef t;              // model time after the step
  float* out;               // [capacity][ncraft][4 + nf]
  unsigned int* count;
  unsigned int capacity;
};

}  // namespace g3m3
