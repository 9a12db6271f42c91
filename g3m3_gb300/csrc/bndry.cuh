// bndry.cuh -- argument blocks of the boundary and nested-grid kernels.
#pragma once

#include "kargs.cuh"

namespace g3m3 {

struct OuterArgs {          // bndry_outer on the outermost box
  float* f[G3M3_NFIELDS];
  const float* b0[3];
  Dims d;
  float rmassq, rmassh, rmasso;
  float srho, rho_frac, o_conc, spress, spx, spy, spz;
  float sbx_wind, sby_wind, sbz_wind, ti_te;
};

struct InnerArgs {          // bndry_inner on box mbndry
  float* f[G3M3_NFIELDS];
  const int* ij[3];         // srf, mid, zero: (mbndry,3,m) column-major
  const float* parm[3];     // (mbndry,7,m)
  int num[3];
  int mbndry, box;
  Dims d;
  float xmin, ymin, dx, dy, re_equiv, v_rot;
  int only;                 // 0: the three lists at once; l + 1: list l alone
  int serial;               // with only: one thread walks the list in order
};

// How the inner-boundary lists of one box must be applied.  The reference
// runs the srf, mid and zero lists one after another, each in order, so a
// cell named twice ends with its last entry's values.  The lists its own
// set-up builds name each cell once; then every entry can run at once.
struct InnerOrder {
  bool overlap = false;                     // a cell in two lists: the lists in turn
  bool repeat[3] = {false, false, false};   // a cell twice in list l: list l in order
  bool any() const { return overlap || repeat[0] || repeat[1] || repeat[2]; }
};

// ij: host copies of the three (mbndry,3,m) lists; entries outside the box
// are skipped by the kernels and ignored here
InnerOrder inner_order(const int* const ij[3], const int num[3], int mbndry, int box, const Dims& d);

enum FlanksMode { FLANKS_PLAIN = 0, FLANKS_KEEP = 1, FLANKS_REUSE = 2 };

struct FlanksArgs {         // fine box shell from the time-interpolated coarse box
  float* target[G3M3_NFIELDS];
  const float* curc[G3M3_NFIELDS];
  const float* oldc[G3M3_NFIELDS];
  int nf;
  int fields_per_block;     // set by the launcher
  int mode;                 // FlanksMode
  long nshell;              // shell cells (set by the launcher)
  float* ibuf;              // interpolated values [field][shell cell] (KEEP / REUSE)
  Dims d;
  ScalarRef t1;             // (t_new(mb)-t)/(t_new(mb)-t_old(mb)) rounded to FP32
  float sxmin, symin, szmin, sx, sy, sz;        // fine box
  float bxmin, bymin, bzmin, delx, dely, delz;  // coarse box
};

struct CorerArgs {          // coarse cells under the fine box from the fine box
  float* coarse[G3M3_NFIELDS];
  const float* fine[G3M3_NFIELDS];
  int nf;
  Dims d;
  int nskip, nbx1, nby1, nbz1;
  int ni, nj, nk;
};

struct SyncedArgs {         // flanks_synced
  float* fine[G3M3_NFIELDS];
  const float* coarse[G3M3_NFIELDS];
  int nf;
  Dims d;
  float sxmin, symin, szmin, sx, sy, sz;
  float bxmin, bymin, bzmin, delx, dely, delz;
  int kb_top, kb_bot, jb_top, jb_bot, ib_top, ib_bot;
};

long shell_count(const Dims& d, int D);
void launch_bndry_outer(const OuterArgs& a, cudaStream_t s);
// returns the number of launches (1, or one per nonempty list when o.any())
int launch_bndry_inner(const InnerArgs& a, const InnerOrder& o, cudaStream_t s);
void launch_flanks(const FlanksArgs& a, cudaStream_t s);
void launch_corer(const CorerArgs& a, cudaStream_t s);
void launch_flanks_synced(const SyncedArgs& a, cudaStream_t s);

}  // namespace g3m3
