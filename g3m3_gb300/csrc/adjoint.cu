// adjoint.cu -- the adjoint of the engine's main steps (g3m3_adjoint_*):
// gradients of a virtual-spacecraft misfit with respect to the upstream
// parameters of bndry_outer's wind face and to the initial state.
//
// Forward (g3m3_adjoint_forward): the model runs N main steps as the engine
// always does (host-launched), with the time-step schedule recorded, the
// state checkpointed every K steps, and the misfit of the samples that fall
// in each main step accumulated at its end.
//
// Backward (g3m3_adjoint_backward), segment by segment from the last: the
// segment's checkpoint is restored and its main steps re-run under the
// recorded schedule with the tape attached, which snapshots, per box-step,
// the box's start state and the state after each stage's boundaries and
// after its guards (the reverses of the linear steps -- flanks, corer, the
// outer boundary's copies -- need no primal values).  Then the main steps of the
// segment are reversed action by action (box-steps, core syncs, final
// syncs, the div B pass), each kernel's reverse (k_adj.cu) reading the
// snapshots.  The time-step schedule is held fixed (its dependence on the
// state through set_speed_agrd's maxima is not differentiated); the div B
// solves are differentiated as exact linear solves, so the gradient is that
// of the converged projection.
#include <chrono>
#include <cstring>
#include <vector>

#include "adjoint.cuh"
#include "model.cuh"

namespace g3m3 {
int cg_begin(g3m3_ctx* c, CgRun& r, float errlim, bool given, int redos0, int hint);
int cg_step(g3m3_ctx* c, CgRun& r, bool* done);
void fill_flanks_geometry(FlanksArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);
void fill_corer_geometry(CorerArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                         const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);
void fill_synced_geometry(SyncedArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);

// One recorded box-step: its scalars and the device snapshots ([34][n3]
// blocks) its reverse reads.
struct BoxRec {
  int box = 0;
  float dt2 = 0, dt = 0, t1p = 0, t1c = 0;
  float* s0 = nullptr;     // state at the start (cur before store_array)
  float* snap[TP_NPOINTS] = {};
};

struct Rec {               // one recorded action, in launch order
  enum Kind { BOX, CORE, FINAL, DIVB } kind;
  int box;
  int boxrec;              // BOX: index into Tape::boxes
  float* snap;             // FINAL: cur of the box after the corer, before set_rho
};

struct Tape {
  std::vector<float*> chunks;   // device arena in chunks, bump-allocated per segment
  std::vector<size_t> chunk_cap;
  size_t chunk_i = 0, chunk_used = 0;
  size_t block = 0;             // floats of one [34][n3] block
  std::vector<BoxRec> boxes;
  std::vector<Rec> acts;
  std::vector<int> step_first;  // first action of each recorded main step
  int err = 0;
  g3m3_ctx* ctx = nullptr;

  void reset() {
    chunk_i = 0;
    chunk_used = 0;
    boxes.clear();
    acts.clear();
    step_first.clear();
    err = 0;
  }
  float* take(size_t n) {
    n = (n + 63) & ~(size_t)63;
    while (chunk_i < chunks.size() && chunk_used + n > chunk_cap[chunk_i]) {
      chunk_i++;
      chunk_used = 0;
    }
    if (chunk_i == chunks.size()) {
      const size_t cap = n > ((size_t)1 << 29) ? n : ((size_t)1 << 29);   // 2 GiB chunks
      float* p = nullptr;
      const cudaError_t e = dev_alloc(ctx, (void**)&p, cap * sizeof(float));
      if (e != cudaSuccess) {
        cudaGetLastError();
        err = cuda_check(ctx, e, "adjoint tape");
        return nullptr;
      }
      chunks.push_back(p);
      chunk_cap.push_back(cap);
      chunk_used = 0;
    }
    float* p = chunks[chunk_i] + chunk_used;
    chunk_used += n;
    return p;
  }
  void free_all() {
    for (float* p : chunks) cudaFree(p);
    chunks.clear();
    chunk_cap.clear();
  }
};

namespace {

inline float* field(g3m3_model* m, int role, int f, int b) { return m->buf[role][f] + (size_t)(b - 1) * m->n3; }
inline float* cur(g3m3_model* m, int f, int b) { return field(m, m->role_cur[b - 1], f, b); }
inline float* old(g3m3_model* m, int f, int b) { return field(m, m->role_old[b - 1], f, b); }
inline float* wrk(g3m3_model* m, int f, int b) { return field(m, 2, f, b); }

void copy_box(g3m3_model* m, float* dst, float* (*get)(g3m3_model*, int, int), int b) {
  const float* src[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) src[q] = get(m, q, b);
  launch_copy_fields(dst, src, G3M3_NFIELDS, m->n3, m->stream);
}

}  // namespace

// ---- tape hooks (the engine calls these while m->tape is set) ----------
void tape_box_start(g3m3_model* m, int box, float dt2, float dt, float t1p, float t1c) {
  Tape& t = *m->tape;
  if (t.err) return;
  BoxRec r;
  r.box = box;
  r.dt2 = dt2; r.dt = dt; r.t1p = t1p; r.t1c = t1c;
  r.s0 = t.take(t.block);
  for (int q = 0; q < TP_NPOINTS; q++) r.snap[q] = t.take(t.block);
  if (t.err) return;
  copy_box(m, r.s0, cur, box);
  t.boxes.push_back(r);
  t.acts.push_back(Rec{Rec::BOX, box, (int)t.boxes.size() - 1, nullptr});
}

void tape_snap(g3m3_model* m, int point, int box, float* const fields[G3M3_NFIELDS]) {
  Tape& t = *m->tape;
  if (t.err || t.boxes.empty() || t.boxes.back().box != box) return;
  const float* src[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) src[q] = fields[q];
  launch_copy_fields(t.boxes.back().snap[point], src, G3M3_NFIELDS, m->n3, m->stream);
}

void tape_core(g3m3_model* m, int box) { m->tape->acts.push_back(Rec{Rec::CORE, box, -1, nullptr}); }

void tape_final(g3m3_model* m, int box) {
  Tape& t = *m->tape;
  float* s = t.take(t.block);
  if (!s) return;
  copy_box(m, s, cur, box);
  t.acts.push_back(Rec{Rec::FINAL, box, -1, s});
}

void tape_divb(g3m3_model* m) { m->tape->acts.push_back(Rec{Rec::DIVB, 0, -1, nullptr}); }

}  // namespace g3m3

using namespace g3m3;

struct g3m3_adjoint {
  g3m3_model* m = nullptr;
  int nsteps = 0, every = 0, nseg = 0;
  float errlim = 0.0f;
  // forward record
  std::vector<double> schedule;        // t_stepnew of every box before each main step
  std::vector<float*> ckpt;            // per segment start, and the end: cur (34 n4) + wrk epres (n4)
  std::vector<double> ck_t;
  std::vector<int> ck_done;
  bool forward_done = false;
  // samples
  int nsamp = 0;
  std::vector<int> samp_step;          // main step (1-based) at whose end each sample is taken
  float* d_xyz = nullptr;              // [nsamp][3]
  float* d_target = nullptr;           // [nsamp][4]
  float* d_resid = nullptr;            // [nsamp][4]
  double* d_loss = nullptr;
  double* h_loss = nullptr;            // pinned
  // adjoint state
  float* a_cur = nullptr;              // [34][n4]
  float* a_old = nullptr;              // [34][n4]
  float* a_we = nullptr;               // [n4]
  float* aW = nullptr;                 // [34][n3]: the wrk buffer of the box-step being reversed
  float* aO = nullptr;                 // [34][n3]: its start state (old)
  float* a_sc = nullptr;               // [19][n3]: efld 3, cur 3, bs 3, btot, ev 3, tv 3, vt 3
  float* p1 = nullptr;                 // [34][n3]
  float* a_p1 = nullptr;               // [34][n3]
  float* fm = nullptr;                 // [3][34][n3] each: flux-correction reverse, per face
  float* fw = nullptr;
  float* fp = nullptr;
  float* glist = nullptr;
  unsigned* gcount = nullptr;
  unsigned gcap = 0;
  float* cgv = nullptr;                // [8][n3]: adjoint div B right-hand side and 7 CG vectors
  CgState* cgst = nullptr;
  CgState* host_cgst = nullptr;        // pinned
  double* d_aparam = nullptr;          // [8]
  Tape tape;
  double phase_s[6] = {};              // last backward: re-run with snapshots, reverse kernels, div B reverse;
                                       // then the host time spent issuing each (before the stream drained)
  bool prof = false;                   // GPU time per stage of the box-step reverses
  cudaEvent_t ev[17] = {};
  double stage_ms[16] = {};
  float* mem = nullptr;
  int64_t cell_updates = 0;
};

namespace {

int adj_err(g3m3_adjoint* a, int code, const char* msg) { return set_err(a->m->ctx, code, "%s", msg); }

float* acur(g3m3_adjoint* a, int f, int b) { return a->a_cur + (size_t)f * a->m->n4 + (size_t)(b - 1) * a->m->n3; }
float* aold(g3m3_adjoint* a, int f, int b) { return a->a_old + (size_t)f * a->m->n4 + (size_t)(b - 1) * a->m->n3; }
float* blk(float* base, int f, size_t n3) { return base + (size_t)f * n3; }

// scratch adjoint slots of the fields stage
enum { SC_EFLD = 0, SC_CUR = 3, SC_BS = 6, SC_BTOT = 9, SC_EV = 10, SC_TV = 13, SC_VT = 16 };
float* sc(g3m3_adjoint* a, int slot) { return a->a_sc + (size_t)slot * a->m->n3; }

Geom box_geom(const g3m3_model* m, int b) {
  Geom g;
  g.xmin = m->p.grd_xmin[b - 1]; g.ymin = m->p.grd_ymin[b - 1]; g.zmin = m->p.grd_zmin[b - 1];
  g.dx = (m->p.grd_xmax[b - 1] - m->p.grd_xmin[b - 1]) / (float)(m->d.nx - 1);
  g.dy = (m->p.grd_ymax[b - 1] - m->p.grd_ymin[b - 1]) / (float)(m->d.ny - 1);
  g.dz = (m->p.grd_zmax[b - 1] - m->p.grd_zmin[b - 1]) / (float)(m->d.nz - 1);
  return g;
}

// guards (set_rho + set_speed_agrd, or set_rho alone) in reverse, in place on a[]
void rev_guard(g3m3_adjoint* A, const float* pre, float* const aa[G3M3_NFIELDS], int b, bool speed) {
  g3m3_model* m = A->m;
  const g3m3_params& p = m->p;
  AdjGuardArgs g{};
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    g.pre[q] = pre + (size_t)q * m->n3;
    g.a[q] = aa[q];
  }
  g.d = m->d;
  g.smallbit = p.smallbit; g.aniso_limit = p.aniso_limit; g.vlim = p.vlim_factor * (float)b;
  g.svlim[0] = p.qvlim; g.svlim[1] = p.hvlim; g.svlim[2] = p.ovlim;
  g.sclim[0] = p.qclim; g.sclim[1] = p.hclim; g.sclim[2] = p.oclim;
  g.cslim = p.cslim; g.iso_flag = m->iso_flag; g.isotropic = p.isotropic != 0;
  g.do_speed = speed ? 1 : 0;
  g.list = A->glist; g.list_count = A->gcount; g.list_cap = A->gcap;
  launch_adj_guard(g, m->stream);
}

// boundaries of a stage in reverse: bndry_inner first (the engine runs it
// after the outer boundary or beside the flanks on disjoint cells), then
// bndry_outer (outermost box) or the flanks at time weight t1
void rev_boundary(g3m3_adjoint* A, const float* post, float* const aa[G3M3_NFIELDS], int b, float t1, bool flanks) {
  g3m3_model* m = A->m;
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  if (b <= p.mbndry && m->inner_set) {
    AdjInnerArgs in{};
    for (int q = 0; q < G3M3_NFIELDS; q++) {
      in.post[q] = post + (size_t)q * m->n3;
      in.a[q] = aa[q];
    }
    const int mb = p.mbndry;
    for (int l = 0; l < 3; l++) {
      in.ij[l] = m->ij[l];
      in.parm[l] = m->parm[l];
      in.num[l] = m->num[l][mb - 1];
    }
    in.mbndry = mb; in.box = mb; in.d = m->d;
    in.dx = (p.grd_xmax[mb - 1] - p.grd_xmin[mb - 1]) / ((float)m->d.nx - 1.0f);
    in.dy = (p.grd_ymax[mb - 1] - p.grd_ymin[mb - 1]) / ((float)m->d.ny - 1.0f);
    in.xmin = p.grd_xmin[mb - 1]; in.ymin = p.grd_ymin[mb - 1];
    in.re_equiv = p.re_equiv; in.v_rot = p.v_rot;
    launch_adj_inner(in, m->stream);
  }
  if (b == ng) {
    AdjOuterArgs o{};
    for (int q = 0; q < G3M3_NFIELDS; q++) {
      o.post[q] = post + (size_t)q * m->n3;
      o.a[q] = aa[q];
    }
    for (int q = 0; q < 3; q++) o.b0[q] = m->b0[q] + (size_t)(b - 1) * m->n3;
    o.a_param = A->d_aparam;
    o.d = m->d;
    o.rmassq = p.rmassq; o.rmassh = p.rmassh; o.rmasso = p.rmasso;
    o.srho = p.srho; o.rho_frac = p.rho_frac; o.o_conc = p.o_conc; o.spress = p.spress;
    o.spx = p.spx; o.spy = p.spy; o.spz = p.spz;
    o.sbx_wind = p.sbx_wind; o.sby_wind = p.sby_wind; o.sbz_wind = p.sbz_wind; o.ti_te = p.ti_te;
    launch_adj_outer(o, m->stream);
  } else if (flanks) {
    FlanksArgs geo{};
    fill_flanks_geometry(geo, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax,
                         p.grd_zmin, p.grd_zmax);
    AdjFlanksArgs f{};
    for (int q = 0; q < G3M3_NFIELDS; q++) {
      f.a_target[q] = aa[q];
      f.a_curc[q] = acur(A, q, b + 1);
      f.a_oldc[q] = aold(A, q, b + 1);
    }
    f.nf = G3M3_NFIELDS; f.d = m->d; f.t1 = t1;
    f.sxmin = geo.sxmin; f.symin = geo.symin; f.szmin = geo.szmin; f.sx = geo.sx; f.sy = geo.sy; f.sz = geo.sz;
    f.bxmin = geo.bxmin; f.bymin = geo.bymin; f.bzmin = geo.bzmin;
    f.delx = geo.delx; f.dely = geo.dely; f.delz = geo.delz;
    launch_adj_flanks(f, m->stream);
  }
}


// the fields stage (calcur, bs/btot, fnd_evel, BandE) of the state `st`
// in reverse: the scratch adjoints go to the state's adjoints `as`; the
// primal scratch is recomputed first
void rev_fields(g3m3_adjoint* A, float* const st[G3M3_NFIELDS], float* const as[G3M3_NFIELDS], int b) {
  g3m3_model* m = A->m;
  const size_t n3 = m->n3;
  engine_fields(m, st, b);
  AdjFieldsArgs f{};
  for (int q = 0; q < 3; q++) {
    f.b[q] = st[G3M3_F_BX + q];
    f.b0[q] = m->b0[q] + (size_t)(b - 1) * n3;
    f.rho[q] = st[10 * q];
    for (int c = 0; c < 3; c++) {
      f.p[q][c] = st[10 * q + 1 + c];
      f.a_p[q][c] = as[10 * q + 1 + c];
    }
    f.cur[q] = m->curr[q]; f.bs[q] = m->bs[q]; f.ev[q] = m->ev[q];
    f.a_efld[q] = sc(A, SC_EFLD + q); f.a_cur[q] = sc(A, SC_CUR + q); f.a_bs[q] = sc(A, SC_BS + q);
    f.a_ev[q] = sc(A, SC_EV + q); f.a_tv[q] = sc(A, SC_TV + q);
    f.a_b[q] = as[G3M3_F_BX + q];
    f.a_rho[q] = as[10 * q];
  }
  f.a_btot = sc(A, SC_BTOT);
  f.epres = st[G3M3_F_EPRES];
  f.a_epres = as[G3M3_F_EPRES];
  const bool resist = b <= m->p.mbndry && m->p.resist < 5000.0f && m->inner_set;
  f.rst_e = resist ? m->rst_e + (size_t)(b - 1) * n3 : nullptr;
  f.d = m->d;
  f.rmass[0] = m->p.rmassq; f.rmass[1] = m->p.rmassh; f.rmass[2] = m->p.rmasso;
  f.reynolds = m->p.reynolds;
  f.rx = f.ry = f.rz = m->p.xspac[b - 1];
  f.smallbit = m->p.smallbit;
  launch_adj_fields(f, m->stream);
}

// a push stage in reverse: out was written from src and old with the
// fields stage's scratch of src (recomputed into the model's scratch first)
void rev_push(g3m3_adjoint* A, float* const src[G3M3_NFIELDS], float* const oldst[G3M3_NFIELDS],
              float* const a_out[G3M3_NFIELDS], float* const a_src[G3M3_NFIELDS], float* const a_old[G3M3_NFIELDS],
              int b, float delt, bool corrector) {
  g3m3_model* m = A->m;
  const float rx = m->p.xspac[b - 1];
  engine_fields(m, src, b);
  AdjPushFieldArgs pf{};
  pf.wrkepres = src[G3M3_F_EPRES];
  for (int q = 0; q < 3; q++) {
    pf.ev[q] = m->ev[q];
    pf.a_ev[q] = sc(A, SC_EV + q);
    pf.a_b[q] = a_out[G3M3_F_BX + q];
    pf.a_oldb[q] = a_old[G3M3_F_BX + q];
    pf.a_efld[q] = sc(A, SC_EFLD + q);
  }
  pf.a_epres = a_out[G3M3_F_EPRES];
  pf.a_wrkepres = a_src[G3M3_F_EPRES];
  pf.a_oldepres = a_old[G3M3_F_EPRES];
  pf.d = m->d; pf.rx = pf.ry = pf.rz = rx; pf.gamma = m->p.gamma; pf.gamma1 = m->p.gamma1; pf.delt = delt;
  // the predictor's push_elec writes cur's epres, which the corrector's
  // overwrites before anything reads it: only the corrector's is reversed
  pf.do_elec = corrector ? 1 : 0;
  pf.do_bfld = 1;
  pf.boundary_from_old = corrector ? 1 : 0;
  launch_adj_push_field(pf, m->stream);
  const float masses[3] = {m->p.rmassq, m->p.rmassh, m->p.rmasso};
  for (int s = 0; s < 3; s++) {
    AdjPushIonArgs a{};
    for (int f = 0; f < 10; f++) {
      a.src[f] = src[10 * s + f];
      a.old[f] = oldst[10 * s + f];
      a.a_out[f] = a_out[10 * s + f];
      a.a_src[f] = a_src[10 * s + f];
      a.a_old[f] = a_old[10 * s + f];
    }
    for (int q = 0; q < 3; q++) {
      a.bs[q] = m->bs[q]; a.efld[q] = m->efld[q]; a.tv[q] = m->tv[q];
      a.a_bs[q] = sc(A, SC_BS + q); a.a_efld[q] = sc(A, SC_EFLD + q); a.a_tv[q] = sc(A, SC_TV + q);
    }
    a.btot = m->btot;
    a.a_btot = sc(A, SC_BTOT);
    a.d = m->d;
    a.g = box_geom(m, b);
    a.rmass = masses[s]; a.grav = m->p.grav; a.re_equiv = m->p.re_equiv; a.reynolds = m->p.reynolds;
    a.delt = delt;
    a.boundary_from_old = corrector ? 1 : 0;
    launch_adj_push_ion(a, m->stream);
  }
}

void rev_corer(g3m3_adjoint* A, int b) {
  g3m3_model* m = A->m;
  const g3m3_params& p = m->p;
  CorerArgs geo{};
  fill_corer_geometry(geo, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax, p.grd_zmin,
                      p.grd_zmax);
  AdjCorerArgs c{};
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    c.a_coarse[q] = acur(A, q, b + 1);
    c.a_fine[q] = acur(A, q, b);
  }
  c.nf = G3M3_NFIELDS; c.d = m->d;
  c.nskip = geo.nskip; c.nbx1 = geo.nbx1; c.nby1 = geo.nby1; c.nbz1 = geo.nbz1;
  c.ni = geo.ni; c.nj = geo.nj; c.nk = geo.nk;
  launch_adj_corer(c, m->stream);
}

// the adjoint solve A z = rhs of one div B projection: the forward's CG on
// the same (symmetric) operator, from z = 0
int solve(g3m3_adjoint* A, int b) {
  g3m3_model* m = A->m;
  const size_t n = m->n3;
  CgRun r;
  DivbArgs& a = r.a;
  a = DivbArgs{};
  a.rhs = A->cgv; a.x = A->cgv + n; a.xs = A->cgv + 2 * n; a.g = A->cgv + 3 * n; a.h = A->cgv + 4 * n;
  a.xi = A->cgv + 5 * n; a.xj = A->cgv + 6 * n;
  a.st = A->cgst; a.d = m->d;
  a.rx = a.ry = a.rz = m->p.xspac[b - 1];
  r.host_st = A->host_cgst;
  r.s = m->stream;
  r.graphs = nullptr;
  launch_zero(a.x, n, m->stream);
  int st = cg_begin(m->ctx, r, A->errlim, true, 1, 16);
  bool done = false;
  while (!st && !done) st = cg_step(m->ctx, r, &done);
  if (st) return st;
  // a zero right-hand side (no adjoint reaches this box's B) has the zero
  // solution; the CG would divide 0 by 0 there
  if (!(A->host_cgst->bsq > 0.0)) launch_zero(a.x, n, m->stream);
  if (r.status == CG_MAXIT) return set_err(m->ctx, G3M3_ERR_NOCONV, "adjoint div B solve: too many iterations");
  return G3M3_OK;
}

int rev_divb(g3m3_adjoint* A) {
  g3m3_model* m = A->m;
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  for (int b = ng - 1; b >= 1; b--) rev_corer(A, b);
  for (int b = 1; b <= ng - 1; b++) {
    SyncedArgs geo{};
    fill_synced_geometry(geo, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax,
                         p.grd_zmin, p.grd_zmax);
    AdjSyncedArgs s{};
    for (int q = 0; q < 3; q++) {
      s.a_fine[q] = acur(A, G3M3_F_BX + q, b);
      s.a_coarse[q] = acur(A, G3M3_F_BX + q, b + 1);
    }
    s.nf = 3; s.d = m->d;
    s.sxmin = geo.sxmin; s.symin = geo.symin; s.szmin = geo.szmin; s.sx = geo.sx; s.sy = geo.sy; s.sz = geo.sz;
    s.bxmin = geo.bxmin; s.bymin = geo.bymin; s.bzmin = geo.bzmin;
    s.delx = geo.delx; s.dely = geo.dely; s.delz = geo.delz;
    s.kb_top = geo.kb_top; s.kb_bot = geo.kb_bot; s.jb_top = geo.jb_top; s.jb_bot = geo.jb_bot;
    s.ib_top = geo.ib_top; s.ib_bot = geo.ib_bot;
    launch_adj_synced(s, m->stream);
  }
  int worst = G3M3_OK;
  for (int b = 1; b <= ng; b++) {
    for (int rep = 0; rep < 2; rep++) {   // the two projections of the box
      AdjDivbArgs d{};
      for (int q = 0; q < 3; q++) d.a_b[q] = acur(A, G3M3_F_BX + q, b);
      d.rhs = A->cgv;
      d.z = A->cgv + m->n3;
      d.d = m->d;
      d.rx = p.xspac[b - 1];
      launch_adj_divb_rhs(d, m->stream);
      const int st = solve(A, b);
      if (st && st != G3M3_ERR_NOCONV) return st;
      if (st) worst = st;
      launch_adj_divb_apply(d, m->stream);
    }
  }
  return worst;
}

void tab_of(float* base, size_t n3, float* t[G3M3_NFIELDS]) {
  for (int q = 0; q < G3M3_NFIELDS; q++) t[q] = base + (size_t)q * n3;
}

// GPU-time marks between the stages of a box-step's reverse (when profiling)
void mark(g3m3_adjoint* A, int k) {
  if (A->prof) cudaEventRecord(A->ev[k], A->m->stream);
}

// one recorded box-step in reverse (the engine's enqueue_box_step read
// backwards; aC is the adjoint of cur, aW of wrk, aO of old = the start state)
void rev_box(g3m3_adjoint* A, const BoxRec& R) {
  g3m3_model* m = A->m;
  const int b = R.box;
  const size_t n3 = m->n3;
  cudaStream_t s = m->stream;
  float *aC[G3M3_NFIELDS], *aW[G3M3_NFIELDS], *aO[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) aC[q] = acur(A, q, b);
  tab_of(A->aW, n3, aW);
  tab_of(A->aO, n3, aO);
  // the adjoints after the box-step: cur's (aC); wrk's, of which only the
  // electron pressure is read later; old's (the start state as the finer
  // box's flanks read it after this step)
  mark(A, 0);
  cudaMemsetAsync(A->aW, 0, (size_t)G3M3_NFIELDS * n3 * sizeof(float), s);
  {
    const float* we = A->a_we + (size_t)(b - 1) * n3;
    launch_copy_fields(aW[G3M3_F_EPRES], &we, 1, n3, s);
    float* src[G3M3_NFIELDS];
    for (int q = 0; q < G3M3_NFIELDS; q++) src[q] = aold(A, q, b);
    launch_move_fields(A->aO, src, G3M3_NFIELDS, n3, s);
  }
  float *s0[G3M3_NFIELDS], *w1[G3M3_NFIELDS], *c1[G3M3_NFIELDS], *l1[G3M3_NFIELDS];
  tab_of(R.s0, n3, s0);
  tab_of(R.snap[TP_PRED_GUARD], n3, w1);
  tab_of(R.snap[TP_CORR_GUARD], n3, c1);
  tab_of(R.snap[TP_LAP_GUARD], n3, l1);
  // flux correction: guards, boundaries, fcsmooth of (wrk, old)
  mark(A, 1);
  rev_guard(A, R.snap[TP_FCS_BNDRY], aC, b, true);
  mark(A, 2);
  rev_boundary(A, R.snap[TP_FCS_BNDRY], aC, b, R.t1c, true);
  {
    AdjFcsArgs f{};
    for (int q = 0; q < G3M3_NFIELDS; q++) {
      f.wrk[q] = l1[q];
      f.old[q] = s0[q];
      f.a_px[q] = aC[q];
      f.a_wrk[q] = aW[q];
      f.a_old[q] = aO[q];
      f.chi[q] = q >= G3M3_F_BX ? m->p.diferg : m->p.difrho;
    }
    f.p1 = A->p1; f.a_p1 = A->a_p1; f.fm = A->fm; f.fw = A->fw; f.fp = A->fp;
    f.nf = G3M3_NFIELDS; f.d = m->d;
    mark(A, 3);
    launch_adj_fcs(f, s);
  }
  // Lapidus: guards, boundaries, the smoothing of the corrector's state
  mark(A, 4);
  rev_guard(A, R.snap[TP_LAP_BNDRY], aW, b, true);
  mark(A, 5);
  rev_boundary(A, R.snap[TP_LAP_BNDRY], aW, b, R.t1c, true);
  for (int sp = 0; sp < 3; sp++) {
    AdjLapArgs l{};
    for (int f = 0; f < 10; f++) {
      l.in[f] = c1[10 * sp + f];
      l.a_out[f] = aW[10 * sp + f];
      l.a_in[f] = aC[10 * sp + f];
      l.chi[f] = f == 0 ? m->p.chirho : m->p.chipxyz;
    }
    l.nf = 10;
    for (int q = 0; q < 3; q++) {
      l.vp[q] = c1[10 * sp + 1 + q];
      l.a_vp[q] = aC[10 * sp + 1 + q];
    }
    l.vrho = c1[10 * sp];
    l.a_vrho = aC[10 * sp];
    l.vfloor = m->p.smallbit; l.delt = R.dt; l.d = m->d;
    launch_adj_lap(l, s);
  }
  engine_vtot(m, c1);   // the primal mass-averaged velocity into the model's scratch
  {
    AdjLapArgs lb{};
    lb.in[0] = c1[G3M3_F_EPRES]; lb.a_out[0] = aW[G3M3_F_EPRES]; lb.a_in[0] = aC[G3M3_F_EPRES];
    lb.chi[0] = m->p.chipxyz;
    for (int q = 0; q < 3; q++) {
      lb.in[1 + q] = c1[G3M3_F_BX + q];
      lb.a_out[1 + q] = aW[G3M3_F_BX + q];
      lb.a_in[1 + q] = aC[G3M3_F_BX + q];
      lb.chi[1 + q] = m->p.chierg;
      lb.v[q] = m->vt[q];
      lb.a_v[q] = sc(A, SC_VT + q);
    }
    lb.nf = 4; lb.delt = R.dt; lb.d = m->d;
    launch_adj_lap(lb, s);
    // the Lapidus reverses only read wrk's adjoint; the corrector's pushes
    // accumulate into it next
    cudaMemsetAsync(A->aW, 0, (size_t)G3M3_NFIELDS * n3 * sizeof(float), s);
    AdjVtotArgs v{};
    for (int sp = 0; sp < 3; sp++) {
      v.rho[sp] = c1[10 * sp];
      v.a_rho[sp] = aC[10 * sp];
      for (int q = 0; q < 3; q++) {
        v.p[sp][q] = c1[10 * sp + 1 + q];
        v.a_p[sp][q] = aC[10 * sp + 1 + q];
      }
    }
    for (int q = 0; q < 3; q++) v.a_v[q] = sc(A, SC_VT + q);
    v.d = m->d;
    mark(A, 6);
    launch_adj_vtot(v, s);
  }
  // corrector: guards; boundaries (its flanks go to wrk, which Lapidus
  // overwrites before any read, so only bndry_inner / bndry_outer on cur
  // are reversed); the pushes from (wrk, old); the fields of wrk
  mark(A, 7);
  rev_guard(A, R.snap[TP_CORR_BNDRY], aC, b, true);
  mark(A, 8);
  rev_boundary(A, R.snap[TP_CORR_BNDRY], aC, b, R.t1c, false);
  mark(A, 9);
  rev_push(A, w1, s0, aC, aW, aO, b, R.dt, true);
  mark(A, 10);
  rev_fields(A, w1, aW, b);
  // predictor: guards, boundaries, the pushes from (old, old), the fields of old
  mark(A, 11);
  rev_guard(A, R.snap[TP_PRED_BNDRY], aW, b, true);
  mark(A, 12);
  rev_boundary(A, R.snap[TP_PRED_BNDRY], aW, b, R.t1p, true);
  mark(A, 13);
  rev_push(A, s0, s0, aW, aO, aO, b, R.dt2, false);
  mark(A, 14);
  rev_fields(A, s0, aO, b);
  // before the box-step: cur held the start state; wrk's epres the value
  // the predictor's push_elec read
  mark(A, 15);
  launch_copy_fields_out(aC, A->aO, G3M3_NFIELDS, n3, s);
  const float* we = aW[G3M3_F_EPRES];
  float* dst = A->a_we + (size_t)(b - 1) * n3;
  launch_copy_fields_out(&dst, we, 1, n3, s);
  mark(A, 16);
  if (A->prof) {
    cudaEventSynchronize(A->ev[16]);
    for (int q = 0; q < 16; q++) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, A->ev[q], A->ev[q + 1]);
      A->stage_ms[q] += ms;
    }
  }
}

void loss_args(g3m3_adjoint* A, LossArgs& L, int first, int count) {
  g3m3_model* m = A->m;
  const g3m3_params& p = m->p;
  L = LossArgs{};
  for (int b = 1; b <= p.n_grids; b++) {
    for (int q = 0; q < 3; q++) {
      L.f[b - 1][q] = cur(m, G3M3_F_BX + q, b);
      L.rho[b - 1][q] = cur(m, 10 * q, b);
      L.a_f[b - 1][q] = acur(A, G3M3_F_BX + q, b);
      L.a_rho[b - 1][q] = acur(A, 10 * q, b);
    }
    L.gmin[3 * (b - 1) + 0] = p.grd_xmin[b - 1]; L.gmax[3 * (b - 1) + 0] = p.grd_xmax[b - 1];
    L.gmin[3 * (b - 1) + 1] = p.grd_ymin[b - 1]; L.gmax[3 * (b - 1) + 1] = p.grd_ymax[b - 1];
    L.gmin[3 * (b - 1) + 2] = p.grd_zmin[b - 1]; L.gmax[3 * (b - 1) + 2] = p.grd_zmax[b - 1];
    L.xspac[b - 1] = p.xspac[b - 1];
  }
  L.xyz = A->d_xyz + 3 * (size_t)first;
  L.target = A->d_target + 4 * (size_t)first;
  L.resid = A->d_resid + 4 * (size_t)first;
  L.loss = A->d_loss;
  L.n = count;
  L.n_grids = p.n_grids;
  L.d = m->d;
  L.re_equiv = p.re_equiv;
}

// samples taken at the end of main step `step` (1-based): [first, first + count)
void samples_of(const g3m3_adjoint* A, int step, int* first, int* count) {
  int f = 0;
  while (f < A->nsamp && A->samp_step[f] < step) f++;
  int c = 0;
  while (f + c < A->nsamp && A->samp_step[f + c] == step) c++;
  *first = f;
  *count = c;
}

int save_ckpt(g3m3_adjoint* A, int i) {
  g3m3_model* m = A->m;
  float* ck = A->ckpt[i];
  for (int f = 0; f < G3M3_NFIELDS; f++)
    for (int b = 1; b <= m->p.n_grids; b++)
      G3M3_CUDA(m->ctx, cudaMemcpyAsync(ck + (size_t)f * m->n4 + (size_t)(b - 1) * m->n3, cur(m, f, b),
                                        m->n3 * sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
  for (int b = 1; b <= m->p.n_grids; b++)
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(ck + (size_t)G3M3_NFIELDS * m->n4 + (size_t)(b - 1) * m->n3,
                                      wrk(m, G3M3_F_EPRES, b), m->n3 * sizeof(float), cudaMemcpyDeviceToDevice,
                                      m->stream));
  A->ck_t[i] = m->t;
  A->ck_done[i] = m->nsteps_done;
  return G3M3_OK;
}

int load_ckpt(g3m3_adjoint* A, int i) {
  g3m3_model* m = A->m;
  const float* ck = A->ckpt[i];
  for (int f = 0; f < G3M3_NFIELDS; f++)
    for (int b = 1; b <= m->p.n_grids; b++)
      G3M3_CUDA(m->ctx, cudaMemcpyAsync(cur(m, f, b), ck + (size_t)f * m->n4 + (size_t)(b - 1) * m->n3,
                                        m->n3 * sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
  for (int b = 1; b <= m->p.n_grids; b++)
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(wrk(m, G3M3_F_EPRES, b),
                                      ck + (size_t)G3M3_NFIELDS * m->n4 + (size_t)(b - 1) * m->n3,
                                      m->n3 * sizeof(float), cudaMemcpyDeviceToDevice, m->stream));
  m->t = A->ck_t[i];
  m->nsteps_done = A->ck_done[i];
  return G3M3_OK;
}

// run main steps [s0, s1) (0-based) under the recorded schedule
int run_forced(g3m3_adjoint* A, int s0, int s1) {
  g3m3_model* m = A->m;
  m->forced_steps = A->schedule.data() + (size_t)s0 * m->p.n_grids;
  m->forced_n = s1 - s0;
  m->forced_i = 0;
  int rc = G3M3_OK;
  for (int st = s0; st < s1 && !rc; st++) {
    if (m->tape) m->tape->step_first.push_back((int)m->tape->acts.size());
    rc = g3m3_model_run(m, 1, 0);
    if (rc == G3M3_ERR_NOCONV) rc = G3M3_OK;   // the reference warns and goes on
    if (!rc && m->tape && m->tape->err) rc = m->tape->err;
  }
  m->forced_steps = nullptr;
  m->forced_n = 0;
  return rc;
}

}  // namespace

extern "C" {

int g3m3_adjoint_create(g3m3_model* m, int nsteps, int checkpoint_every, float cg_errlim, g3m3_adjoint** out) {
  if (!m || !out || nsteps < 1 || checkpoint_every < 1) return G3M3_ERR_ARG;
  *out = nullptr;
  if (m->p.mbndry != 1) return set_err(m->ctx, G3M3_ERR_ARG, "adjoint: mbndry must be 1");
  if (m->inner_set && !m->lists_unique)
    return set_err(m->ctx, G3M3_ERR_ARG, "adjoint: inner-boundary lists must name distinct cells");
  g3m3_adjoint* A = new g3m3_adjoint();
  A->m = m;
  A->nsteps = nsteps;
  A->every = checkpoint_every;
  A->nseg = (nsteps + checkpoint_every - 1) / checkpoint_every;
  A->errlim = cg_errlim > 0.0f ? cg_errlim : m->p.divb_errlim;
  A->tape.ctx = m->ctx;
  A->tape.block = (size_t)G3M3_NFIELDS * m->n3;
  const size_t n3 = m->n3, n4 = m->n4;
  A->gcap = (unsigned)(3 * n3 < 0xffffffffu ? 3 * n3 : 0xffffffffu);
  const size_t nface = 3 * (size_t)G3M3_NFIELDS * n3;
  const size_t floats = 2 * (size_t)G3M3_NFIELDS * n4 + n4 + 2 * (size_t)G3M3_NFIELDS * n3 + 19 * n3 +
                        2 * (size_t)G3M3_NFIELDS * n3 + (size_t)A->gcap * 11 + 8 * n3 + 3 * nface +
                        (size_t)(A->nseg + 1) * (G3M3_NFIELDS + 1) * n4;
  cudaError_t e = dev_alloc(m->ctx, (void**)&A->mem, floats * sizeof(float));
  if (e != cudaSuccess) {
    delete A;
    return cuda_check(m->ctx, e, "adjoint");
  }
  float* q = A->mem;
  A->a_cur = q; q += (size_t)G3M3_NFIELDS * n4;
  A->a_old = q; q += (size_t)G3M3_NFIELDS * n4;
  A->a_we = q; q += n4;
  A->aW = q; q += (size_t)G3M3_NFIELDS * n3;
  A->aO = q; q += (size_t)G3M3_NFIELDS * n3;
  A->a_sc = q; q += 19 * n3;
  A->p1 = q; q += (size_t)G3M3_NFIELDS * n3;
  A->a_p1 = q; q += (size_t)G3M3_NFIELDS * n3;
  A->glist = q; q += (size_t)A->gcap * 11;
  A->cgv = q; q += 8 * n3;
  A->fm = q; q += nface;
  A->fw = q; q += nface;
  A->fp = q; q += nface;
  for (int i = 0; i <= A->nseg; i++) {
    A->ckpt.push_back(q);
    q += (size_t)(G3M3_NFIELDS + 1) * n4;
  }
  A->ck_t.assign(A->nseg + 1, 0.0);
  A->ck_done.assign(A->nseg + 1, 0);
  int rc = G3M3_OK;
  if ((e = dev_alloc(m->ctx, (void**)&A->gcount, 64)) != cudaSuccess ||
      (e = dev_alloc(m->ctx, (void**)&A->cgst, sizeof(CgState))) != cudaSuccess ||
      (e = dev_alloc(m->ctx, (void**)&A->d_aparam, 8 * sizeof(double))) != cudaSuccess ||
      (e = dev_alloc(m->ctx, (void**)&A->d_loss, sizeof(double))) != cudaSuccess ||
      (e = cudaMallocHost(&A->host_cgst, sizeof(CgState))) != cudaSuccess ||
      (e = cudaMallocHost(&A->h_loss, sizeof(double))) != cudaSuccess)
    rc = cuda_check(m->ctx, e, "adjoint");
  if (!rc) {
    e = cudaMemsetAsync(A->a_sc, 0, 19 * n3 * sizeof(float), m->stream);
    if (e != cudaSuccess) rc = cuda_check(m->ctx, e, "adjoint");
  }
  if (rc) {
    g3m3_adjoint_destroy(A);
    return rc;
  }
  *out = A;
  return G3M3_OK;
}

int g3m3_adjoint_destroy(g3m3_adjoint* A) {
  if (!A) return G3M3_ERR_ARG;
  cudaStreamSynchronize(A->m->stream);
  A->tape.free_all();
  cudaFree(A->mem);
  cudaFree(A->gcount);
  cudaFree(A->cgst);
  cudaFree(A->d_aparam);
  cudaFree(A->d_loss);
  cudaFree(A->d_xyz);
  cudaFree(A->d_target);
  cudaFree(A->d_resid);
  if (A->host_cgst) cudaFreeHost(A->host_cgst);
  if (A->h_loss) cudaFreeHost(A->h_loss);
  for (int q = 0; q < 17; q++)
    if (A->ev[q]) cudaEventDestroy(A->ev[q]);
  delete A;
  return G3M3_OK;
}

int g3m3_adjoint_set_samples(g3m3_adjoint* A, int n, const float* xyz, const int* step, const float* target) {
  if (!A || n < 0 || (n > 0 && (!xyz || !step || !target))) return G3M3_ERR_ARG;
  g3m3_model* m = A->m;
  for (int i = 0; i < n; i++)
    if (step[i] < 1 || step[i] > A->nsteps || (i > 0 && step[i] < step[i - 1]))
      return set_err(m->ctx, G3M3_ERR_ARG, "adjoint samples: steps must be in 1..%d and non-decreasing", A->nsteps);
  cudaFree(A->d_xyz); cudaFree(A->d_target); cudaFree(A->d_resid);
  A->d_xyz = A->d_target = A->d_resid = nullptr;
  A->nsamp = n;
  A->samp_step.assign(step, step + n);
  if (n == 0) return G3M3_OK;
  cudaError_t e;
  if ((e = dev_alloc(m->ctx, (void**)&A->d_xyz, 3 * (size_t)n * sizeof(float))) != cudaSuccess ||
      (e = dev_alloc(m->ctx, (void**)&A->d_target, 4 * (size_t)n * sizeof(float))) != cudaSuccess ||
      (e = dev_alloc(m->ctx, (void**)&A->d_resid, 4 * (size_t)n * sizeof(float))) != cudaSuccess)
    return cuda_check(m->ctx, e, "adjoint samples");
  G3M3_CUDA(m->ctx, cudaMemcpyAsync(A->d_xyz, xyz, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  G3M3_CUDA(m->ctx, cudaMemcpyAsync(A->d_target, target, 4 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice,
                                    m->stream));
  G3M3_CUDA(m->ctx, cudaStreamSynchronize(m->stream));
  return G3M3_OK;
}

int g3m3_adjoint_forward(g3m3_adjoint* A, const double* schedule_in, double* loss) {
  if (!A) return G3M3_ERR_ARG;
  g3m3_model* m = A->m;
  const int ng = m->p.n_grids;
  A->schedule.assign((size_t)A->nsteps * ng, 0.0);
  G3M3_CUDA(m->ctx, cudaMemsetAsync(A->d_loss, 0, sizeof(double), m->stream));
  int rc = G3M3_OK;
  for (int st = 0; st < A->nsteps && !rc; st++) {
    if (st % A->every == 0 && (rc = save_ckpt(A, st / A->every))) break;
    if (schedule_in) {
      std::memcpy(A->schedule.data() + (size_t)st * ng, schedule_in + (size_t)st * ng, ng * sizeof(double));
      rc = run_forced(A, st, st + 1);
    } else {
      std::memcpy(A->schedule.data() + (size_t)st * ng, m->t_stepnew, ng * sizeof(double));
      rc = g3m3_model_run(m, 1, 0);
      if (rc == G3M3_ERR_NOCONV) rc = G3M3_OK;
    }
    if (rc) break;
    int first, count;
    samples_of(A, st + 1, &first, &count);
    if (count) {
      LossArgs L;
      loss_args(A, L, first, count);
      launch_loss(L, m->stream, false);
    }
  }
  if (!rc) rc = save_ckpt(A, A->nseg);
  if (rc) return rc;
  G3M3_CUDA(m->ctx, cudaMemcpyAsync(A->h_loss, A->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  G3M3_CUDA(m->ctx, cudaStreamSynchronize(m->stream));
  if (loss) *loss = *A->h_loss;
  A->forward_done = true;
  return G3M3_OK;
}

int g3m3_adjoint_schedule(g3m3_adjoint* A, double* out) {
  if (!A || !out || !A->forward_done) return G3M3_ERR_ARG;
  std::memcpy(out, A->schedule.data(), A->schedule.size() * sizeof(double));
  return G3M3_OK;
}

int g3m3_adjoint_backward(g3m3_adjoint* A, double* grad_params, float* grad_state, float* grad_wrk_epres) {
  if (!A) return G3M3_ERR_ARG;
  g3m3_model* m = A->m;
  if (!A->forward_done) return set_err(m->ctx, G3M3_ERR_STATE, "adjoint: backward before forward");
  const size_t n4 = m->n4;
  cudaStream_t s = m->stream;
  G3M3_CUDA(m->ctx, cudaMemsetAsync(A->a_cur, 0, (2 * (size_t)G3M3_NFIELDS * n4 + n4) * sizeof(float), s));
  G3M3_CUDA(m->ctx, cudaMemsetAsync(A->d_aparam, 0, 8 * sizeof(double), s));
  int rc = G3M3_OK;
  int worst = G3M3_OK;
  for (double& t : A->phase_s) t = 0.0;
  using clk = std::chrono::steady_clock;
  auto lap = [&](clk::time_point& t0, int phase) {   // phase time, the stream drained
    const clk::time_point tq = clk::now();
    cudaStreamSynchronize(s);
    const clk::time_point t1 = clk::now();
    A->phase_s[phase] += std::chrono::duration<double>(t1 - t0).count();
    A->phase_s[3 + phase] += std::chrono::duration<double>(tq - t0).count();
    t0 = t1;
  };
  clk::time_point t0 = clk::now();
  for (int seg = A->nseg - 1; seg >= 0 && !rc; seg--) {
    const int s0 = seg * A->every;
    const int s1 = s0 + A->every < A->nsteps ? s0 + A->every : A->nsteps;
    if ((rc = load_ckpt(A, seg))) break;
    A->tape.reset();
    m->tape = &A->tape;
    rc = run_forced(A, s0, s1);
    m->tape = nullptr;
    if (rc) break;
    lap(t0, 0);
    const Tape& T = A->tape;
    for (int st = s1 - 1; st >= s0 && !rc; st--) {
      const int k = st - s0;
      // the misfit of the samples at the end of this step, taken from the
      // state the step left (its cur buffers)
      int first, count;
      samples_of(A, st + 1, &first, &count);
      if (count) {
        LossArgs L;
        loss_args(A, L, first, count);
        launch_loss(L, s, true);
      }
      const int a0 = T.step_first[k];
      const int a1 = k + 1 < (int)T.step_first.size() ? T.step_first[k + 1] : (int)T.acts.size();
      for (int ai = a1 - 1; ai >= a0 && !rc; ai--) {
        const Rec& R = T.acts[ai];
        switch (R.kind) {
          case Rec::BOX: rev_box(A, T.boxes[R.boxrec]); break;
          case Rec::CORE: rev_corer(A, R.box); break;
          case Rec::FINAL: {
            float* aC[G3M3_NFIELDS];
            for (int q = 0; q < G3M3_NFIELDS; q++) aC[q] = acur(A, q, R.box);
            rev_guard(A, R.snap, aC, R.box, false);
            rev_corer(A, R.box);
            break;
          }
          case Rec::DIVB: {
            lap(t0, 1);
            const int st2 = rev_divb(A);
            if (st2 == G3M3_ERR_NOCONV) worst = st2;
            else rc = st2;
            lap(t0, 2);
            break;
          }
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_check(m->ctx, e, "adjoint");
      }
    }
    lap(t0, 1);
  }
  // leave the model at the end of the run, as the forward did
  if (!rc) rc = load_ckpt(A, A->nseg);
  if (rc) return rc;
  if (grad_params) G3M3_CUDA(m->ctx, cudaMemcpyAsync(grad_params, A->d_aparam, 8 * sizeof(double),
                                                     cudaMemcpyDeviceToHost, s));
  if (grad_state)
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(grad_state, A->a_cur, (size_t)G3M3_NFIELDS * n4 * sizeof(float),
                                      cudaMemcpyDefault, s));
  if (grad_wrk_epres)
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(grad_wrk_epres, A->a_we, n4 * sizeof(float), cudaMemcpyDefault, s));
  G3M3_CUDA(m->ctx, cudaStreamSynchronize(s));
  return worst;
}

int g3m3_adjoint_profile(g3m3_adjoint* A, int on, double* stage_ms) {
  if (!A) return G3M3_ERR_ARG;
  if (stage_ms)
    for (int q = 0; q < 16; q++) stage_ms[q] = A->stage_ms[q];
  for (int q = 0; q < 16; q++) A->stage_ms[q] = 0.0;
  if (on && !A->ev[0])
    for (int q = 0; q < 17; q++) G3M3_CUDA(A->m->ctx, cudaEventCreate(&A->ev[q]));
  A->prof = on != 0;
  return G3M3_OK;
}

int g3m3_adjoint_phases(g3m3_adjoint* A, double* seconds) {
  if (!A || !seconds) return G3M3_ERR_ARG;
  for (int q = 0; q < 6; q++) seconds[q] = A->phase_s[q];
  return G3M3_OK;
}

size_t g3m3_adjoint_tape_bytes(g3m3_adjoint* A) {
  if (!A) return 0;
  size_t b = 0;
  for (size_t c : A->tape.chunk_cap) b += c * sizeof(float);
  return b;
}

}  // extern "C"
