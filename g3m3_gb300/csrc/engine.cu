// engine.cu -- the multi-box step engine (g3m3_model_*): the reference's
// main time loop (3d_main.f90:1925-3095) on device-resident state.
//
// Differences in mechanism (not in results) from the reference loop:
//  * store_array (old <- cur, 34 copies per box-step, :2193-2229) is a
//    rotation of the cur/old buffer roles.  Until the corrector writes cur,
//    every read of cur is served from old (which then holds the same
//    values), and the corrector pushes write the boundary cells of cur from
//    old, so cur ends the push with the bits the reference has.
//  * set_rho + set_speed_agrd run as one fused pass (k_guards.cu).
//  * bs/btot are produced by the calcur kernel; BandE is one launch.
//  * the time-dependent scalars of a main step (dt/2, dt, flank time
//    weights) live in a small device table, so that one captured CUDA graph
//    replays every main step with the same schedule shape.
#include <array>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <map>
#include <cstdio>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "model.cuh"

namespace g3m3 {
int run_divb(g3m3_ctx* c, float* bx, float* by, float* bz, const Dims& d, float rx, float errlim, CgState* st,
             CgState* host_st, float* vec, cudaStream_t s, int* iters_out);
int cg_begin(g3m3_ctx* c, CgRun& r, float errlim, bool given, int redos0, int hint);
int cg_step(g3m3_ctx* c, CgRun& r, bool* done);
void fill_flanks_geometry(FlanksArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);
void fill_corer_geometry(CorerArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                         const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);
void fill_synced_geometry(SyncedArgs& a, int nx, int ny, int nz, int box, const float* gxmin, const float* gxmax,
                          const float* gymin, const float* gymax, const float* gzmin, const float* gzmax);
void launch_bande_interior(const BandEArgs& a, cudaStream_t s);
}  // namespace g3m3

using namespace g3m3;

namespace {

// NVTX ranges around the stages of a box-step, the main step and the div B
// pass, so that a profiler can attribute host-launched kernels to them (in
// a replayed graph the kernels carry the range of the replay).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

const char* const kBoxStepRange[8] = {"box-step 1", "box-step 2", "box-step 3", "box-step 4",
                                      "box-step 5", "box-step 6", "box-step 7", "box-step 8+"};

}  // namespace


namespace {

inline float* F(g3m3_model* m, int role, int f, int box) { return m->buf[role][f] + (size_t)(box - 1) * m->n3; }
inline float* C(g3m3_model* m, int f, int b) { return F(m, m->role_cur[b - 1], f, b); }
inline float* O(g3m3_model* m, int f, int b) { return F(m, m->role_old[b - 1], f, b); }
inline float* W(g3m3_model* m, int f, int b) { return F(m, 2, f, b); }

using Getter = float* (*)(g3m3_model*, int, int);

int scal_slot(g3m3_model* m, float v) {
  if (m->nscal >= m->scal_cap) return -1;
  m->h_scal[m->nscal] = v;
  return m->nscal++;
}

ScalarRef sref(g3m3_model* m, int slot) { return ScalarRef{m->h_scal[slot], m->d_scal + slot}; }

cudaStream_t S(g3m3_model* m) { return m->stream; }

// Independent kernels of a stage run on side streams: fork orders the side
// streams after the work already queued on the model's stream, join orders
// the model's stream after the side streams' work.  In a captured step the
// pairs become parallel branches of the graph.
void fork_aux(g3m3_model* m) {
  cudaEventRecord(m->fork_ev, S(m));
  for (int i = 0; i < 3; i++) cudaStreamWaitEvent(m->aux[i], m->fork_ev, 0);
}

void join_aux(g3m3_model* m) {
  for (int i = 0; i < 3; i++) {
    cudaEventRecord(m->join_ev[i], m->aux[i]);
    cudaStreamWaitEvent(S(m), m->join_ev[i], 0);
  }
}

void fields_stage(g3m3_model* m, Getter src, int b) {
  const float rx = m->p.xspac[b - 1];
  CurrentArgs ca{};
  for (int q = 0; q < 3; q++) {
    ca.b[q] = src(m, G3M3_F_BX + q, b);
    ca.b0[q] = m->b0[q] + (size_t)(b - 1) * m->n3;
    ca.cur[q] = m->curr[q];
    ca.bs[q] = m->bs[q];
  }
  ca.btot = m->btot;
  ca.d = m->d; ca.rx = rx; ca.ry = rx; ca.rz = rx; ca.smallbit = m->p.smallbit;
  launch_current(ca, S(m));
  EvelArgs ea{};
  for (int s = 0; s < 3; s++) {
    for (int q = 0; q < 3; q++) ea.p[s][q] = src(m, 10 * s + 1 + q, b);
    ea.rho[s] = src(m, 10 * s, b);
  }
  for (int q = 0; q < 3; q++) { ea.cur[q] = m->curr[q]; ea.ev[q] = m->ev[q]; ea.tv[q] = m->tv[q]; }
  ea.d = m->d;
  ea.rmass[0] = m->p.rmassq; ea.rmass[1] = m->p.rmassh; ea.rmass[2] = m->p.rmasso;
  ea.reynolds = m->p.reynolds;
  launch_evel(ea, S(m));
  BandEArgs ba{};
  for (int q = 0; q < 3; q++) {
    ba.efld[q] = m->efld[q]; ba.bs[q] = m->bs[q]; ba.cur[q] = m->curr[q]; ba.ev[q] = m->ev[q];
    ba.rho[q] = src(m, 10 * q, b);
  }
  ba.epres = src(m, G3M3_F_EPRES, b);
  const bool resist = b <= m->p.mbndry && m->p.resist < 5000.0f && m->inner_set;
  ba.rst_e = (resist && m->lists_unique) ? m->rst_e + (size_t)(b - 1) * m->n3 : nullptr;
  ba.d = m->d;
  ba.rmass[0] = m->p.rmassq; ba.rmass[1] = m->p.rmassh; ba.rmass[2] = m->p.rmasso;
  ba.reynolds = m->p.reynolds; ba.rx = rx; ba.ry = rx; ba.rz = rx;
  if (resist && !m->lists_unique) {
    // lists with repeated cells: keep the reference's sequential scatter
    launch_bande_interior(ba, S(m));
    BandEListArgs l{};
    for (int q = 0; q < 3; q++) { l.efld[q] = ba.efld[q]; l.cur[q] = ba.cur[q]; l.rho[q] = ba.rho[q]; l.rmass[q] = ba.rmass[q]; }
    l.rst = m->resistive + (size_t)(b - 1) * m->n3;
    l.mbndry = m->p.mbndry; l.box = b; l.d = m->d;
    for (int q = 1; q < 3; q++) {
      l.ij = m->ij[q];
      l.count = m->num[q][b - 1];
      l.serial = m->inner_order[b - 1].repeat[q] ? 1 : 0;
      launch_bande_list(l, S(m));
    }
    launch_bande_faces(ba.efld, m->d, S(m));
    m->launches_in_step += 3;
  } else {
    launch_bande(ba, S(m));
  }
  m->launches_in_step += 3;
}

void push_stage(g3m3_model* m, Getter out, Getter src, int b, int slot_dt, bool out_is_cur) {
  const float rx = m->p.xspac[b - 1];
  PushFieldArgs pa{};
  pa.wrkepres = W(m, G3M3_F_EPRES, b);
  pa.oldepres = O(m, G3M3_F_EPRES, b);
  pa.epres = C(m, G3M3_F_EPRES, b);
  for (int q = 0; q < 3; q++) {
    pa.ev[q] = m->ev[q];
    pa.b[q] = out(m, G3M3_F_BX + q, b);
    pa.oldb[q] = O(m, G3M3_F_BX + q, b);
    pa.efld[q] = m->efld[q];
  }
  pa.d = m->d; pa.rx = rx; pa.ry = rx; pa.rz = rx; pa.gamma = m->p.gamma; pa.gamma1 = m->p.gamma1;
  pa.delt = sref(m, slot_dt);
  pa.do_elec = 1; pa.do_bfld = 1;
  // cur's boundary must be the start-of-step state (see the file comment);
  // epres always goes to cur, B goes to out
  pa.boundary_from_old = 1;
  // the field push and the three species write disjoint arrays from the
  // same inputs: the species run beside it on the side streams
  fork_aux(m);
  if (!out_is_cur) {
    // predictor: only epres lands in cur; B goes to wrk, whose boundary the
    // reference leaves alone -- run the two pushes separately
    PushFieldArgs e = pa;
    e.do_bfld = 0;
    launch_push_field(e, S(m));
    PushFieldArgs bb = pa;
    bb.do_elec = 0;
    bb.boundary_from_old = 0;
    launch_push_field(bb, S(m));
    m->launches_in_step += 2;
  } else {
    launch_push_field(pa, S(m));
    m->launches_in_step += 1;
  }
  const float masses[3] = {m->p.rmassq, m->p.rmassh, m->p.rmasso};
  for (int s = 0; s < 3; s++) {
    PushIonArgs a{};
    for (int f = 0; f < 10; f++) {
      a.out[f] = out(m, 10 * s + f, b);
      a.old[f] = O(m, 10 * s + f, b);
      a.src[f] = src(m, 10 * s + f, b);
    }
    for (int q = 0; q < 3; q++) { a.bs[q] = m->bs[q]; a.efld[q] = m->efld[q]; a.tv[q] = m->tv[q]; }
    a.btot = m->btot;
    a.d = m->d;
    a.g.xmin = m->p.grd_xmin[b - 1]; a.g.ymin = m->p.grd_ymin[b - 1]; a.g.zmin = m->p.grd_zmin[b - 1];
    a.g.dx = (m->p.grd_xmax[b - 1] - m->p.grd_xmin[b - 1]) / (float)(m->d.nx - 1);
    a.g.dy = (m->p.grd_ymax[b - 1] - m->p.grd_ymin[b - 1]) / (float)(m->d.ny - 1);
    a.g.dz = (m->p.grd_zmax[b - 1] - m->p.grd_zmin[b - 1]) / (float)(m->d.nz - 1);
    a.rmass = masses[s]; a.grav = m->p.grav; a.re_equiv = m->p.re_equiv; a.reynolds = m->p.reynolds;
    a.delt = sref(m, slot_dt);
    a.boundary_from_old = out_is_cur ? 1 : 0;
    a.contracted = m->contracted;
    launch_push_ion(a, m->aux[s]);
    m->launches_in_step += 1;
  }
  join_aux(m);
}

void inner_stage(g3m3_model* m, Getter target, cudaStream_t st) {
  const g3m3_params& p = m->p;
  InnerArgs a{};
  const int mb = p.mbndry;   // bndry_inner always works on box mbndry
  for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = target(m, q, mb);
  for (int l = 0; l < 3; l++) {
    a.ij[l] = m->ij[l];
    a.parm[l] = m->parm[l];
    a.num[l] = m->num[l][mb - 1];
  }
  a.mbndry = mb; a.box = mb; a.d = m->d;
  a.dx = (p.grd_xmax[mb - 1] - p.grd_xmin[mb - 1]) / ((float)m->d.nx - 1.0f);
  a.dy = (p.grd_ymax[mb - 1] - p.grd_ymin[mb - 1]) / ((float)m->d.ny - 1.0f);
  a.xmin = p.grd_xmin[mb - 1]; a.ymin = p.grd_ymin[mb - 1];
  a.re_equiv = p.re_equiv; a.v_rot = p.v_rot;
  m->launches_in_step += launch_bndry_inner(a, m->inner_order[mb - 1], st);
}

void boundary_stage(g3m3_model* m, Getter target, int b, int slot_t1, Getter inner_target = nullptr,
                    int flank_mode = FLANKS_PLAIN) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  // bndry_inner's cells lie deep inside the box, the flank shell on its
  // faces: with both, bndry_inner runs beside the flanks on a side stream
  const bool side = b < ng && b <= p.mbndry && m->inner_set && !m->inner_in_shell;
  if (side) {
    fork_aux(m);
    inner_stage(m, inner_target ? inner_target : target, m->aux[0]);
  }
  if (b == ng) {
    OuterArgs a{};
    for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = target(m, q, b);
    for (int q = 0; q < 3; q++) a.b0[q] = m->b0[q] + (size_t)(b - 1) * m->n3;
    a.d = m->d;
    a.rmassq = p.rmassq; a.rmassh = p.rmassh; a.rmasso = p.rmasso;
    a.srho = p.srho; a.rho_frac = p.rho_frac; a.o_conc = p.o_conc; a.spress = p.spress;
    a.spx = p.spx; a.spy = p.spy; a.spz = p.spz;
    a.sbx_wind = p.sbx_wind; a.sby_wind = p.sby_wind; a.sbz_wind = p.sbz_wind; a.ti_te = p.ti_te;
    launch_bndry_outer(a, S(m));
  } else {
    FlanksArgs a{};
    for (int q = 0; q < G3M3_NFIELDS; q++) {
      a.target[q] = target(m, q, b);
      a.curc[q] = C(m, q, b + 1);
      a.oldc[q] = O(m, q, b + 1);
    }
    a.nf = G3M3_NFIELDS;
    a.mode = flank_mode;
    a.ibuf = m->flank_ibuf;
    fill_flanks_geometry(a, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax,
                         p.grd_zmin, p.grd_zmax);
    a.t1 = sref(m, slot_t1);
    launch_flanks(a, S(m));
  }
  m->launches_in_step += 1;
  if (side) join_aux(m);
  else if (b <= p.mbndry && m->inner_set) inner_stage(m, inner_target ? inner_target : target, S(m));
}

// set_rho and set_speed_agrd; maxima go to the box's slot when `record`
int guard_stage(g3m3_model* m, Getter target, int b, bool speed, bool record) {
  const g3m3_params& p = m->p;
  GuardArgs a{};
  for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = target(m, q, b);
  for (int q = 0; q < 3; q++) a.b0[q] = m->b0[q] + (size_t)(b - 1) * m->n3;
  a.btot = m->btot;
  a.d = m->d;
  a.smallbit = p.smallbit; a.aniso_limit = p.aniso_limit; a.vlim = p.vlim_factor * (float)b;
  a.svlim[0] = p.qvlim; a.svlim[1] = p.hvlim; a.svlim[2] = p.ovlim;
  a.sclim[0] = p.qclim; a.sclim[1] = p.hclim; a.sclim[2] = p.oclim;
  a.cslim = p.cslim; a.iso_flag = m->iso_flag; a.isotropic = p.isotropic != 0;
  a.do_set_rho = 1; a.do_speed = speed ? 1 : 0;
  a.list = m->glist; a.list_cap = (unsigned)m->gcap; a.list_count = m->words;
  a.maxbits = record ? m->words + 8 + 5 * (b - 1) : m->words + 1;
  const size_t zero_bytes = 6 * sizeof(unsigned);
  cudaError_t e = cudaMemsetAsync(m->words, 0, zero_bytes, S(m));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "memset guard words");
  if (record) {
    e = cudaMemsetAsync(m->words + 8 + 5 * (b - 1), 0, 5 * sizeof(unsigned), S(m));
    if (e != cudaSuccess) return cuda_check(m->ctx, e, "memset box maxima");
  }
  launch_guards(a, S(m));
  m->launches_in_step += 1;
  if (speed) {
    ScatterArgs sa{};
    for (int q = 0; q < G3M3_NFIELDS; q++) sa.f[q] = a.f[q];
    sa.list = m->glist; sa.list_count = m->words; sa.list_cap = (unsigned)m->gcap;
    launch_guard_scatter(sa, S(m));
    m->launches_in_step += 1;
  }
  return G3M3_OK;
}

void corer_stage(g3m3_model* m, int b) {
  const g3m3_params& p = m->p;
  CorerArgs a{};
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    a.fine[q] = C(m, q, b);
    a.coarse[q] = C(m, q, b + 1);
  }
  a.nf = G3M3_NFIELDS;
  fill_corer_geometry(a, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax, p.grd_zmin,
                      p.grd_zmax);
  launch_corer(a, S(m));
  m->launches_in_step += 1;
}

float flank_t1(g3m3_model* m, int b, double t_grid) {
  const int mb = b + 1;
  return (float)((m->t_new[mb - 1] - t_grid) / (m->t_new[mb - 1] - m->t_old[mb - 1]));
}

// One entry of a main step's plan.
struct Action {
  enum Kind { BOX_STEP, CORE_SYNC, FINAL_SYNC } kind;
  int box;
  int s_half, s_full, s_t1p, s_t1c;   // scalar-table slots
};

// Host-only: the reference's schedule for one main step (3d_main.f90:
// 1929-1968, 2142-2165, 3044-3095).  Advances the host time bookkeeping,
// fills the scalar table and returns the actions in launch order.
int plan_main_step(g3m3_model* m, std::vector<Action>& acts) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  acts.clear();
  m->nscal = 0;
  if (m->forced_steps && m->forced_i < m->forced_n) {   // a prescribed schedule (the adjoint's fixed dt)
    for (int b = 0; b < ng; b++) m->t_stepnew[b] = m->forced_steps[(size_t)m->forced_i * ng + b];
    m->forced_i++;
  }
  double smallest_step = 0.0;
  int m_smallest = ng;
  for (int box = ng; box >= 1; box--) {
    m->t_step[box - 1] = m->t_stepnew[box - 1];
    m->t_old[box - 1] = 0.0;
    m->t_new[box - 1] = 0.0;
    if (box == ng) {
      smallest_step = m->t_step[box - 1];
      m_smallest = box;
    } else {
      if (m->t_step[box - 1] > m->t_step[box]) m->t_step[box - 1] = m->t_step[box];
      if (smallest_step > m->t_step[box - 1]) {
        smallest_step = m->t_step[box - 1];
        m_smallest = box;
      }
    }
  }
  for (int box = 1; box <= ng; box++) {
    if (box <= m_smallest) {
      m->t_step[box - 1] = smallest_step;
    } else {
      const float astep = (float)(m->t_step[box - 1] / m->t_step[box - 2] + 0.50);
      int nsteps = (int)astep;
      if (nsteps > 2) nsteps = 2;
      if (nsteps < 1) nsteps = 1;
      m->t_step[box - 1] = m->t_step[box - 2] * nsteps;
    }
  }
  const int m_step = (int)(m->t_step[ng - 1] / m->t_step[m_smallest - 1]);
  const float delt_main = (float)m->t_step[ng - 1];
  if (!(delt_main >= p.t_step_min))
    return set_err(m->ctx, G3M3_ERR_STATE, "main time step %g below t_step_min", (double)delt_main);
  m->t = m->t + (double)delt_main;
  for (int ms = 1; ms <= m_step; ms++) {
    for (int b = ng; b >= 1; b--) {
      bool yes = b == 1;
      if (!yes && m->t_old[b - 1] == m->t_new[b - 1] && m->t_new[b - 1] < m->t_step[ng - 1] &&
          std::fabs(m->t_new[b - 1] - m->t_new[0]) <= (double)0.005f * m->t_step[0])
        yes = true;
      if (!yes) continue;
      Action a{Action::BOX_STEP, b, -1, -1, -1, -1};
      m->t_old[b - 1] = m->t_new[b - 1];
      m->t_new[b - 1] = m->t_old[b - 1] + m->t_step[b - 1];
      const float delt = (float)m->t_step[b - 1];
      const float delt2 = delt / 2.0f;
      a.s_half = scal_slot(m, 0.5f * delt);
      a.s_full = scal_slot(m, delt);
      if (b < ng) {
        double tg = m->t_old[b - 1] + (double)delt2;
        if (tg > m->t_new[b]) tg = m->t_new[b];
        if (tg < m->t_old[b]) tg = m->t_old[b];
        a.s_t1p = scal_slot(m, flank_t1(m, b, tg));
        tg = m->t_old[b - 1] + (double)delt;
        if (tg > m->t_new[b]) tg = m->t_new[b];
        if (tg < m->t_old[b]) tg = m->t_old[b];
        a.s_t1c = scal_slot(m, flank_t1(m, b, tg));
        if (a.s_t1p < 0 || a.s_t1c < 0) return set_err(m->ctx, G3M3_ERR_STATE, "scalar table full");
      }
      if (a.s_half < 0 || a.s_full < 0) return set_err(m->ctx, G3M3_ERR_STATE, "scalar table full");
      acts.push_back(a);
      m->cell_updates += (int64_t)m->n3;
      if (b < ng && std::fabs(m->t_new[b - 1] - m->t_new[b]) <= (double)0.005f * m->t_step[b - 1]) {
        acts.push_back(Action{Action::CORE_SYNC, b, -1, -1, -1, -1});
        m->t_old[b] = m->t_new[b];
      }
    }
  }
  m->t_old[0] = m->t_new[0];
  for (int b = 1; b <= ng - 1; b++) {
    acts.push_back(Action{Action::FINAL_SYNC, b, -1, -1, -1, -1});
    if (b > 1) {  // the reference reads t_old(0) for box 1 (3d_main.f90:3093)
      m->t_old[b - 1] = m->t_old[b - 2];
      m->t_new[b - 1] = m->t_new[b - 2];
    }
  }
  return G3M3_OK;
}

std::string plan_key(g3m3_model* m, const std::vector<Action>& acts) {
  std::string k;
  for (int b = 0; b < m->p.n_grids; b++) k += char('0' + m->role_cur[b]);
  k += ':';
  for (const Action& a : acts) {
    k += a.kind == Action::BOX_STEP ? 's' : (a.kind == Action::CORE_SYNC ? 'c' : 'f');
    k += std::to_string(a.box);
  }
  return k;
}

void apply_role_swaps(g3m3_model* m, const std::vector<Action>& acts) {
  for (const Action& a : acts)
    if (a.kind == Action::BOX_STEP) std::swap(m->role_cur[a.box - 1], m->role_old[a.box - 1]);
}

// The fields stage (calcur, bs/btot, fnd_evel, BandE into the model's
// scratch) and fnd_vtot of an explicit field table, for the adjoint's
// recomputation of primal values.
thread_local float* const* tl_table = nullptr;
float* table_get(g3m3_model*, int f, int) { return tl_table[f]; }

}  // namespace

namespace g3m3 {
void engine_fields(g3m3_model* m, float* const f[G3M3_NFIELDS], int b) {
  tl_table = f;
  fields_stage(m, table_get, b);
  tl_table = nullptr;
}

void engine_vtot(g3m3_model* m, float* const f[G3M3_NFIELDS]) {
  VtotArgs va{};
  for (int s = 0; s < 3; s++) {
    for (int q = 0; q < 3; q++) va.p[s][q] = f[10 * s + 1 + q];
    va.rho[s] = f[10 * s];
  }
  for (int q = 0; q < 3; q++) va.v[q] = m->vt[q];
  va.d = m->d;
  launch_vtot(va, S(m));
}
}  // namespace g3m3

namespace {

// The tape's snapshot of state `get` of box b at `point` (adjoint recording).
void snap(g3m3_model* m, int point, Getter get, int b) {
  if (!m->tape) return;
  float* f[G3M3_NFIELDS];
  for (int q = 0; q < G3M3_NFIELDS; q++) f[q] = get(m, q, b);
  tape_snap(m, point, b, f);
}

// Launch the kernels of one box-step (predictor, corrector, Lapidus, flux
// correction, each followed by boundaries and guards; 3d_main.f90:2170-3039).
int enqueue_box_step(g3m3_model* m, const Action& act) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids, b = act.box;
  Range box_range(kBoxStepRange[b - 1 < 8 ? b - 1 : 7]);
  if (m->tape)
    tape_box_start(m, b, m->h_scal[act.s_half], m->h_scal[act.s_full], act.s_t1p >= 0 ? m->h_scal[act.s_t1p] : 0.0f,
                   act.s_t1c >= 0 ? m->h_scal[act.s_t1c] : 0.0f);
  std::swap(m->role_cur[b - 1], m->role_old[b - 1]);   // store_array
  int st;
  {
    // predictor (reads of cur are served from old, which holds the same data)
    Range r("predictor");
    fields_stage(m, O, b);
    push_stage(m, W, O, b, act.s_half, false);
    boundary_stage(m, W, b, act.s_t1p);
    snap(m, TP_PRED_BNDRY, W, b);
    if ((st = guard_stage(m, W, b, true, false))) return st;
    snap(m, TP_PRED_GUARD, W, b);
  }
  {
    Range r("corrector");
    fields_stage(m, W, b);
    push_stage(m, C, W, b, act.s_full, true);
    if (b == ng) {
      boundary_stage(m, C, b, -1);
    } else {
      // the reference applies the corrector's flanks to the wrk arrays
      // (3d_main.f90:2599-2637) and bndry_inner to cur (:2640-2658).  The
      // coarse box stays fixed through this box-step, so the interpolated
      // flank values at the corrector's time are kept for the two later
      // stages, which use the same time weight.
      boundary_stage(m, W, b, act.s_t1c, C, FLANKS_KEEP);
    }
    snap(m, TP_CORR_BNDRY, C, b);
    if ((st = guard_stage(m, C, b, true, false))) return st;
    snap(m, TP_CORR_GUARD, C, b);
  }
  {
    // Lapidus smoothing (3d_main.f90:2690-2772): the three species beside
    // the electron-pressure and B chain, each writing its own wrk arrays
    Range r("lapidus");
    fork_aux(m);
    for (int s = 0; s < 3; s++) {
      LapArgs la{};
      for (int f = 0; f < 10; f++) {
        la.in[f] = C(m, 10 * s + f, b);
        la.out[f] = W(m, 10 * s + f, b);
        la.chi[f] = f == 0 ? p.chirho : p.chipxyz;
      }
      la.nf = 10;
      for (int q = 0; q < 3; q++) la.vp[q] = C(m, 10 * s + 1 + q, b);
      la.vrho = C(m, 10 * s, b);
      la.vfloor = p.smallbit;
      la.d = m->d;
      la.delt = sref(m, act.s_full);
      launch_lap(la, m->aux[s]);
    }
    VtotArgs va{};
    for (int s = 0; s < 3; s++) {
      for (int q = 0; q < 3; q++) va.p[s][q] = C(m, 10 * s + 1 + q, b);
      va.rho[s] = C(m, 10 * s, b);
    }
    for (int q = 0; q < 3; q++) va.v[q] = m->vt[q];
    va.d = m->d;
    launch_vtot(va, S(m));
    LapArgs lb{};
    lb.in[0] = C(m, G3M3_F_EPRES, b); lb.out[0] = W(m, G3M3_F_EPRES, b); lb.chi[0] = p.chipxyz;
    for (int q = 0; q < 3; q++) {
      lb.in[1 + q] = C(m, G3M3_F_BX + q, b);
      lb.out[1 + q] = W(m, G3M3_F_BX + q, b);
      lb.chi[1 + q] = p.chierg;
      lb.v[q] = m->vt[q];
    }
    lb.nf = 4; lb.d = m->d; lb.delt = sref(m, act.s_full);
    launch_lap(lb, S(m));
    join_aux(m);
    m->launches_in_step += 5;
    boundary_stage(m, W, b, act.s_t1c, nullptr, FLANKS_REUSE);
    snap(m, TP_LAP_BNDRY, W, b);
    if ((st = guard_stage(m, W, b, true, false))) return st;
    snap(m, TP_LAP_GUARD, W, b);
  }
  // flux correction (3d_main.f90:2896-3036)
  Range r("flux_correct");
  FcsArgs fa{};
  for (int q = 0; q < G3M3_NFIELDS; q++) {
    fa.px[q] = C(m, q, b);
    fa.old[q] = O(m, q, b);
    fa.wrk[q] = W(m, q, b);
    fa.chi[q] = q >= G3M3_F_BX ? p.diferg : p.difrho;
  }
  fa.nf = G3M3_NFIELDS; fa.d = m->d; fa.variant = m->fcs_variant;
  launch_fcsmooth(fa, S(m));
  m->launches_in_step += 1;
  boundary_stage(m, C, b, act.s_t1c, nullptr, FLANKS_REUSE);
  snap(m, TP_FCS_BNDRY, C, b);
  return guard_stage(m, C, b, true, true);
}

// the model stream waits for box b's upload before its first use in a
// host-fed step
int upload_wait(g3m3_model* m, int b) {
  if (!m->up_src || b < 1 || b > m->p.n_grids || m->up_waited[b - 1]) return G3M3_OK;
  G3M3_CUDA(m->ctx, cudaStreamWaitEvent(S(m), m->up_ev[b - 1], 0));
  m->up_waited[b - 1] = true;
  return G3M3_OK;
}

int enqueue_plan(g3m3_model* m, const std::vector<Action>& acts) {
  for (const Action& a : acts) {
    int st = G3M3_OK;
    // an action reads box a.box and the coarser box a.box+1; the box-steps
    // of boxes up to mbndry also run bndry_inner on box mbndry
    if ((st = upload_wait(m, a.box)) || (st = upload_wait(m, a.box + 1))) return st;
    if (a.box <= m->p.mbndry && (st = upload_wait(m, m->p.mbndry))) return st;
    switch (a.kind) {
      case Action::BOX_STEP: st = enqueue_box_step(m, a); break;
      case Action::CORE_SYNC:
        if (m->tape) tape_core(m, a.box);
        corer_stage(m, a.box);
        break;
      case Action::FINAL_SYNC:
        corer_stage(m, a.box);
        if (m->tape) tape_final(m, a.box);
        st = guard_stage(m, C, a.box, false, false);
        break;
    }
    if (st) return st;
  }
  return G3M3_OK;
}

// t_stepnew(box) from the recorded maxima (3d_main.f90:3038-3039)
void finish_steps(g3m3_model* m, int box_lo, int box_hi) {
  for (int b = box_lo; b <= box_hi; b++) {
    const unsigned* w = m->host_words + 8 + 5 * (b - 1);
    float v[5];
    for (int q = 0; q < 5; q++) std::memcpy(&v[q], &w[q], sizeof(float));
    float fastest = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3] + v[4] * v[4]);
    fastest = 0.0f > fastest ? 0.0f : fastest;
    const float a = m->p.stepsz * m->p.xspac[b - 1] / fastest;
    m->t_stepnew[b - 1] = (double)(a < m->p.t_step_max ? a : m->p.t_step_max);
  }
}

int alloc_model(g3m3_model* m) {
  const size_t n3 = m->n3, n4 = m->n4;
  const int mb = m->p.mbndry;
  size_t total = 3 * G3M3_NFIELDS * n4 + 3 * n4 + 2 * (size_t)mb * n3 + 19 * n3 + 7 * n3;
  cudaError_t e = dev_alloc(m->ctx, (void**)&m->mem, total * sizeof(float));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "cudaMalloc(model)");
  e = cudaMemsetAsync(m->mem, 0, total * sizeof(float), S(m));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "memset(model)");
  float* q = m->mem;
  for (int r = 0; r < 3; r++)
    for (int f = 0; f < G3M3_NFIELDS; f++) { m->buf[r][f] = q; q += n4; }
  for (int c = 0; c < 3; c++) { m->b0[c] = q; q += n4; }
  m->resistive = q; q += (size_t)mb * n3;
  m->rst_e = q; q += (size_t)mb * n3;
  float** scr[19] = {&m->efld[0], &m->efld[1], &m->efld[2], &m->curr[0], &m->curr[1], &m->curr[2],
                     &m->bs[0],   &m->bs[1],   &m->bs[2],   &m->btot,    &m->ev[0],   &m->ev[1],
                     &m->ev[2],   &m->tv[0],   &m->tv[1],   &m->tv[2],   &m->vt[0],   &m->vt[1],
                     &m->vt[2]};
  for (int i = 0; i < 19; i++) { *scr[i] = q; q += n3; }
  m->cgvec = q; q += 7 * n3;
  m->gcap = 3 * n3;
  e = dev_alloc(m->ctx, (void**)&m->glist, m->gcap * 11 * sizeof(float));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "cudaMalloc(limiter list)");
  e = dev_alloc(m->ctx, (void**)&m->flank_ibuf, (size_t)G3M3_NFIELDS * shell_count(m->d, 2) * sizeof(float));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "cudaMalloc(flank values)");
  const size_t nwords = 8 + 5 * (size_t)G3M3_MAX_GRIDS;
  if ((e = dev_alloc(m->ctx, (void**)&m->words, nwords * sizeof(unsigned))) != cudaSuccess) return cuda_check(m->ctx, e, "words");
  if ((e = cudaMemsetAsync(m->words, 0, nwords * sizeof(unsigned), S(m))) != cudaSuccess)
    return cuda_check(m->ctx, e, "words");
  if ((e = cudaMallocHost(&m->host_words, nwords * sizeof(unsigned))) != cudaSuccess)
    return cuda_check(m->ctx, e, "host words");
  if ((e = dev_alloc(m->ctx, (void**)&m->cg, sizeof(CgState))) != cudaSuccess) return cuda_check(m->ctx, e, "cg");
  if ((e = cudaMallocHost(&m->host_cg, sizeof(CgState))) != cudaSuccess) return cuda_check(m->ctx, e, "cg");
  m->scal_cap = 4096;
  if ((e = dev_alloc(m->ctx, (void**)&m->d_scal, m->scal_cap * sizeof(float))) != cudaSuccess) return cuda_check(m->ctx, e, "scal");
  if ((e = cudaMallocHost(&m->h_scal, m->scal_cap * sizeof(float))) != cudaSuccess)
    return cuda_check(m->ctx, e, "scal");
  for (int b = 0; b < G3M3_MAX_GRIDS; b++) { m->role_cur[b] = 0; m->role_old[b] = 1; }
  return G3M3_OK;
}

struct Roles { int cur[G3M3_MAX_GRIDS], old[G3M3_MAX_GRIDS]; };

Roles save_roles(const g3m3_model* m) {
  Roles r;
  std::memcpy(r.cur, m->role_cur, sizeof r.cur);
  std::memcpy(r.old, m->role_old, sizeof r.old);
  return r;
}

void restore_roles(g3m3_model* m, const Roles& r) {
  std::memcpy(m->role_cur, r.cur, sizeof r.cur);
  std::memcpy(m->role_old, r.old, sizeof r.old);
}

// Host part of a main step: the schedule and scalar table, and the key of
// the step's launch sequence (buffer roles + actions).
int step_plan(g3m3_model* m, std::vector<Action>& acts, std::string& key) {
  const std::string roles = plan_key(m, {});
  int rc = plan_main_step(m, acts);
  if (rc) return rc;
  key = roles + plan_key(m, acts).substr(m->p.n_grids + 1);
  // the step's time for the spacecraft records (t advanced by the plan)
  m->craft_t_slot = m->craft_cap > 0 ? scal_slot(m, (float)m->t) : -1;
  return G3M3_OK;
}

// Device part of a main step on the model's stream: scalar upload, the
// kernels, the read-back of the recorded maxima.  Advances the buffer roles.
int step_enqueue(g3m3_model* m, const std::vector<Action>& acts) {
  const size_t nwords = 8 + 5 * (size_t)G3M3_MAX_GRIDS;
  cudaError_t e;
  m->launches_in_step = 0;
  if ((e = cudaMemcpyAsync(m->d_scal, m->h_scal, m->scal_cap * sizeof(float), cudaMemcpyHostToDevice, S(m))) !=
      cudaSuccess)
    return cuda_check(m->ctx, e, "scalar upload");
  if (m->up_src) {
    // host-fed step: each box's current state on the copy stream, coarsest
    // box first (the order the step first touches them), one event per box
    const int ng = m->p.n_grids;
    G3M3_CUDA(m->ctx, cudaEventRecord(m->up_fork, S(m)));
    G3M3_CUDA(m->ctx, cudaStreamWaitEvent(m->copy_stream, m->up_fork, 0));
    for (int b = ng; b >= 1; b--) {
      for (int f = 0; f < G3M3_NFIELDS; f++)
        G3M3_CUDA(m->ctx, cudaMemcpyAsync(C(m, f, b), m->up_src + (size_t)f * m->n4 + (size_t)(b - 1) * m->n3,
                                          m->n3 * sizeof(float), cudaMemcpyHostToDevice, m->copy_stream));
      G3M3_CUDA(m->ctx, cudaEventRecord(m->up_ev[b - 1], m->copy_stream));
      m->up_waited[b - 1] = false;
    }
  }
  if (m->flux_cap > 0) {
    for (int b = m->p.n_grids; b >= 1; b--)
      if (int st = upload_wait(m, b)) return st;
    // flux_counter of every box at the start of the main step (3d_main.f90:1997-2011)
    for (int b = m->p.n_grids; b >= 1; b--) {
      FluxArgs fa{};
      for (int sp = 0; sp < 3; sp++)
        for (int q = 0; q < 3; q++) fa.p[sp][q] = C(m, 10 * sp + 1 + q, b);
      fa.d = m->d;
      fa.rmass[0] = m->p.rmassq; fa.rmass[1] = m->p.rmassh; fa.rmass[2] = m->p.rmasso;
      fa.grid_spacing = m->flux_scale[b - 1];
      fa.out = m->flux_hist; fa.count = m->flux_count; fa.capacity = (unsigned)m->flux_cap;
      fa.n_grids = m->p.n_grids; fa.box = b; fa.advance = b == 1;
      launch_flux_counter(fa, S(m));
    }
    m->launches_in_step += m->p.n_grids;
  }
  int rc = enqueue_plan(m, acts);
  if (rc) return rc;
  for (int b = 1; b <= m->p.n_grids; b++)   // every upload joins the model stream
    if ((rc = upload_wait(m, b))) return rc;
  if (m->craft_cap > 0 && m->craft_t_slot >= 0) {
    // virtual spacecraft at the end of the step (cft_craft_handling.f90:120-200)
    CraftArgs ca{};
    const g3m3_params& p = m->p;
    ca.geo.n_grids = p.n_grids; ca.geo.d = m->d; ca.geo.re_equiv = p.re_equiv;
    for (int b = 0; b < p.n_grids; b++) {
      ca.geo.gmin[3 * b] = p.grd_xmin[b]; ca.geo.gmin[3 * b + 1] = p.grd_ymin[b]; ca.geo.gmin[3 * b + 2] = p.grd_zmin[b];
      ca.geo.gmax[3 * b] = p.grd_xmax[b]; ca.geo.gmax[3 * b + 1] = p.grd_ymax[b]; ca.geo.gmax[3 * b + 2] = p.grd_zmax[b];
      ca.geo.xspac[b] = p.xspac[b];
    }
    ca.traj = m->craft_traj; ca.start = m->craft_start; ca.ncraft = m->ncraft; ca.nf = m->craft_nf;
    for (int f = 0; f < m->craft_nf; f++)
      for (int b = 1; b <= p.n_grids; b++) ca.fld[f][b - 1] = C(m, m->craft_fields[f], b);
    ca.t = sref(m, m->craft_t_slot);
    ca.out = m->craft_out; ca.count = m->craft_count; ca.capacity = (unsigned)m->craft_cap;
    launch_craft(ca, S(m));
    m->launches_in_step += 1;
  }
  if ((e = cudaMemcpyAsync(m->host_words, m->words, nwords * sizeof(unsigned), cudaMemcpyDeviceToHost, S(m))) !=
      cudaSuccess)
    return cuda_check(m->ctx, e, "readback");
  return G3M3_OK;
}

// After the step's work completed: next time steps, div B when due.
// With `due`, the pass is left to the caller and *due says whether one is
// due now.
int step_finish(g3m3_model* m, bool* due = nullptr) {
  cudaError_t e;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_check(m->ctx, e, "main step");
  finish_steps(m, 1, m->p.n_grids);
  m->nsteps_done += 1;
  const bool now = m->p.divb_every > 0 && (m->nsteps_done % m->p.divb_every) == 0;
  if (due) {
    *due = now;
    return G3M3_OK;
  }
  if (now) {
    const int st = g3m3_model_divb_all(m);
    if (st && st != G3M3_ERR_NOCONV) return st;
    if ((e = cudaStreamSynchronize(S(m))) != cudaSuccess) return cuda_check(m->ctx, e, "divb");
  }
  return G3M3_OK;
}

int copy_in(g3m3_model* m, float* dst, const float* src, size_t n) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(float), cudaMemcpyDefault, S(m));
  return e == cudaSuccess ? G3M3_OK : cuda_check(m->ctx, e, "cudaMemcpyAsync");
}

}  // namespace

extern "C" {

int g3m3_model_create(g3m3_ctx* ctx, const g3m3_params* p, g3m3_model** out) {
  if (!ctx || !p || !out) return G3M3_ERR_ARG;
  *out = nullptr;
  if (p->nx < 5 || p->ny < 5 || p->nz < 5 || p->n_grids < 1 || p->n_grids > G3M3_MAX_GRIDS || p->mbndry < 1 ||
      p->mbndry > p->n_grids)
    return set_err(ctx, G3M3_ERR_ARG, "bad model dimensions");
  g3m3_model* m = new g3m3_model();
  m->ctx = ctx;
  m->stream = ctx->stream;
  m->p = *p;
  {
    cudaError_t e = cudaEventCreateWithFlags(&m->fork_ev, cudaEventDisableTiming);
    for (int i = 0; i < 3 && e == cudaSuccess; i++) {
      e = cudaStreamCreateWithFlags(&m->aux[i], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->join_ev[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
      const int rc = cuda_check(ctx, e, "model streams");
      g3m3_model_destroy(m);
      return rc;
    }
  }
  m->d = Dims{p->nx, p->ny, p->nz};
  m->n3 = m->d.cells();
  m->n4 = m->n3 * p->n_grids;
  int st = alloc_model(m);
  if (st) {
    g3m3_model_destroy(m);
    return st;
  }
  *out = m;
  return G3M3_OK;
}

int g3m3_model_destroy(g3m3_model* m) {
  if (!m) return G3M3_ERR_ARG;
  cudaStreamSynchronize(S(m));
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  if (m->mem) cudaFree(m->mem);
  if (m->glist) cudaFree(m->glist);
  if (m->flank_ibuf) cudaFree(m->flank_ibuf);
  if (m->words) cudaFree(m->words);
  if (m->host_words) cudaFreeHost(m->host_words);
  if (m->cg) cudaFree(m->cg);
  if (m->host_cg) cudaFreeHost(m->host_cg);
  if (m->cg_box) cudaFree(m->cg_box);
  if (m->host_cg_box) cudaFreeHost(m->host_cg_box);
  if (m->cgvec_more) cudaFree(m->cgvec_more);
  for (int b = 0; b < G3M3_MAX_GRIDS; b++) {
    if (m->divb_stream[b]) cudaStreamDestroy(m->divb_stream[b]);
    if (m->divb_ev[b]) cudaEventDestroy(m->divb_ev[b]);
    if (m->up_ev[b]) cudaEventDestroy(m->up_ev[b]);
  }
  if (m->copy_stream) cudaStreamDestroy(m->copy_stream);
  if (m->up_fork) cudaEventDestroy(m->up_fork);
  if (m->d_scal) cudaFree(m->d_scal);
  if (m->h_scal) cudaFreeHost(m->h_scal);
  for (int l = 0; l < 3; l++) {
    if (m->ij[l]) cudaFree(m->ij[l]);
    if (m->parm[l]) cudaFree(m->parm[l]);
  }
  if (m->flux_hist) cudaFree(m->flux_hist);
  if (m->flux_count) cudaFree(m->flux_count);
  if (m->craft_traj) cudaFree(m->craft_traj);
  if (m->craft_start) cudaFree(m->craft_start);
  if (m->craft_out) cudaFree(m->craft_out);
  if (m->craft_count) cudaFree(m->craft_count);
  for (int i = 0; i < 3; i++) {
    if (m->aux[i]) cudaStreamDestroy(m->aux[i]);
    if (m->join_ev[i]) cudaEventDestroy(m->join_ev[i]);
  }
  if (m->fork_ev) cudaEventDestroy(m->fork_ev);
  if (m->own_stream) cudaStreamDestroy(m->stream);
  delete m;
  return G3M3_OK;
}

void* g3m3_model_stream(g3m3_model* m) { return m ? (void*)S(m) : nullptr; }

int g3m3_model_set_field(g3m3_model* m, int which, int field, const float* data) {
  if (!m || !data || field < 0 || field >= G3M3_NFIELDS || which < 0 || which > 2) return G3M3_ERR_ARG;
  if (!finite_ok(m->ctx, data, m->n4))
    return set_err(m->ctx, G3M3_ERR_NONFINITE, "field %d holds NaN or Inf", field);
  // `which` names the logical copy; every box shares the same role mapping
  // only before the first step, so per-box roles are honoured here
  for (int b = 1; b <= m->p.n_grids; b++) {
    float* dst = which == 0 ? C(m, field, b) : (which == 1 ? O(m, field, b) : W(m, field, b));
    int st = copy_in(m, dst, data + (size_t)(b - 1) * m->n3, m->n3);
    if (st) return st;
  }
  return G3M3_OK;
}

int g3m3_model_get_field(g3m3_model* m, int which, int field, float* data) {
  if (!m || !data || field < 0 || field >= G3M3_NFIELDS || which < 0 || which > 2) return G3M3_ERR_ARG;
  for (int b = 1; b <= m->p.n_grids; b++) {
    const float* src = which == 0 ? C(m, field, b) : (which == 1 ? O(m, field, b) : W(m, field, b));
    cudaError_t e = cudaMemcpyAsync(data + (size_t)(b - 1) * m->n3, src, m->n3 * sizeof(float), cudaMemcpyDefault,
                                    S(m));
    if (e != cudaSuccess) return cuda_check(m->ctx, e, "get_field");
  }
  cudaError_t e = cudaStreamSynchronize(S(m));
  return e == cudaSuccess ? G3M3_OK : cuda_check(m->ctx, e, "get_field sync");
}

int g3m3_model_set_state(g3m3_model* m, const float* data) {
  if (!m || !data) return G3M3_ERR_ARG;
  for (int f = 0; f < G3M3_NFIELDS; f++) {
    int st = g3m3_model_set_field(m, 0, f, data + (size_t)f * m->n4);
    if (st) return st;
  }
  return G3M3_OK;
}

int g3m3_model_get_state(g3m3_model* m, float* data) {
  if (!m || !data) return G3M3_ERR_ARG;
  for (int f = 0; f < G3M3_NFIELDS; f++)
    for (int b = 1; b <= m->p.n_grids; b++) {
      cudaError_t e = cudaMemcpyAsync(data + (size_t)f * m->n4 + (size_t)(b - 1) * m->n3, C(m, f, b),
                                      m->n3 * sizeof(float), cudaMemcpyDefault, S(m));
      if (e != cudaSuccess) return cuda_check(m->ctx, e, "get_state");
    }
  cudaError_t e = cudaStreamSynchronize(S(m));
  return e == cudaSuccess ? G3M3_OK : cuda_check(m->ctx, e, "get_state sync");
}

int g3m3_model_set_wind(g3m3_model* m, const float* wind) {
  if (!m || !wind) return G3M3_ERR_ARG;
  m->p.srho = wind[0]; m->p.spx = wind[1]; m->p.spy = wind[2]; m->p.spz = wind[3];
  m->p.spress = wind[4]; m->p.sbx_wind = wind[5]; m->p.sby_wind = wind[6]; m->p.sbz_wind = wind[7];
  // captured step graphs hold the old values in their bndry_outer launches
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  m->kernel_nodes.clear();
  return G3M3_OK;
}

int g3m3_model_set_b0(g3m3_model* m, const float* bx0, const float* by0, const float* bz0) {
  if (!m || !bx0 || !by0 || !bz0) return G3M3_ERR_ARG;
  const float* s[3] = {bx0, by0, bz0};
  for (int q = 0; q < 3; q++) {
    int st = copy_in(m, m->b0[q], s[q], m->n4);
    if (st) return st;
  }
  return G3M3_OK;
}

int g3m3_model_set_inner(g3m3_model* m, const float* resistive, const int* ijsrf, const int* numsrf,
                         const float* parm_srf, int msrf, const int* ijmid, const int* nummid, const float* parm_mid,
                         int mmid, const int* ijzero, const int* numzero, const float* parm_zero, int mzero) {
  if (!m || !resistive || !ijsrf || !numsrf || !parm_srf || !ijmid || !nummid || !parm_mid || !ijzero || !numzero ||
      !parm_zero || msrf < 1 || mmid < 1 || mzero < 1)
    return G3M3_ERR_ARG;
  const int mb = m->p.mbndry;
  const int* ij[3] = {ijsrf, ijmid, ijzero};
  const int* num[3] = {numsrf, nummid, numzero};
  const float* parm[3] = {parm_srf, parm_mid, parm_zero};
  const int ml[3] = {msrf, mmid, mzero};
  cudaError_t e;
  for (int l = 0; l < 3; l++) {
    for (int b = 0; b < mb; b++) {
      if (num[l][b] < 0 || num[l][b] > ml[l]) return set_err(m->ctx, G3M3_ERR_ARG, "inner list count out of range");
      m->num[l][b] = num[l][b];
    }
    m->mlen[l] = ml[l];
    if (m->ij[l]) cudaFree(m->ij[l]);
    if (m->parm[l]) cudaFree(m->parm[l]);
    m->ij[l] = nullptr;
    m->parm[l] = nullptr;
    if ((e = dev_alloc(m->ctx, (void**)&m->ij[l], (size_t)mb * 3 * ml[l] * sizeof(int))) != cudaSuccess)
      return cuda_check(m->ctx, e, "lists");
    if ((e = dev_alloc(m->ctx, (void**)&m->parm[l], (size_t)mb * 7 * ml[l] * sizeof(float))) != cudaSuccess)
      return cuda_check(m->ctx, e, "parms");
    if ((e = cudaMemcpy(m->ij[l], ij[l], (size_t)mb * 3 * ml[l] * sizeof(int), cudaMemcpyDefault)) != cudaSuccess)
      return cuda_check(m->ctx, e, "lists");
    if ((e = cudaMemcpy(m->parm[l], parm[l], (size_t)mb * 7 * ml[l] * sizeof(float), cudaMemcpyDefault)) !=
        cudaSuccess)
      return cuda_check(m->ctx, e, "parms");
    m->h_ij[l].assign(ij[l], ij[l] + (size_t)mb * 3 * ml[l]);
    if (l == 0) m->inner_in_shell = false;
    for (int b = 0; b < mb; b++)
      for (int n = 0; n < num[l][b]; n++) {
        const int i = ij[l][b + (size_t)mb * (0 + 3 * (size_t)n)];
        const int j = ij[l][b + (size_t)mb * (1 + 3 * (size_t)n)];
        const int k = ij[l][b + (size_t)mb * (2 + 3 * (size_t)n)];
        if (i <= 2 || j <= 2 || k <= 2 || i >= m->d.nx - 1 || j >= m->d.ny - 1 || k >= m->d.nz - 1)
          m->inner_in_shell = true;
      }
    m->h_parm[l].resize((size_t)mb * 7 * ml[l]);
    if ((e = cudaMemcpy(m->h_parm[l].data(), parm[l], m->h_parm[l].size() * sizeof(float), cudaMemcpyDefault)) !=
        cudaSuccess)
      return cuda_check(m->ctx, e, "parms");
  }
  // BandE's per-cell resistive coefficient: rst at the ijmid and ijzero
  // cells (sub_BandE.f90:191-219), 0 elsewhere
  std::vector<float> rst((size_t)mb * m->n3), rste((size_t)mb * m->n3, 0.0f);
  std::vector<unsigned char> seen((size_t)mb * m->n3, 0);
  if ((e = cudaMemcpy(rst.data(), resistive, rst.size() * sizeof(float), cudaMemcpyDefault)) != cudaSuccess)
    return cuda_check(m->ctx, e, "resistive");
  m->lists_unique = true;
  for (int b = 1; b <= mb; b++) {
    const int* hp[3] = {ij[0], ij[1], ij[2]};
    const int nb[3] = {m->num[0][b - 1], m->num[1][b - 1], m->num[2][b - 1]};
    m->inner_order[b - 1] = inner_order(hp, nb, mb, b, m->d);
    if (m->inner_order[b - 1].any()) m->lists_unique = false;   // applied in the reference's order
  }
  for (int b = 1; b <= mb; b++)
    for (int l = 1; l < 3; l++)
      for (int n = 0; n < m->num[l][b - 1]; n++) {
        const int i = ij[l][(b - 1) + (size_t)mb * (0 + 3 * (size_t)n)];
        const int j = ij[l][(b - 1) + (size_t)mb * (1 + 3 * (size_t)n)];
        const int k = ij[l][(b - 1) + (size_t)mb * (2 + 3 * (size_t)n)];
        if (i < 2 || j < 2 || k < 2 || i >= m->d.nx || j >= m->d.ny || k >= m->d.nz) {
          m->lists_unique = false;   // a boundary cell: keep the reference's order
          continue;
        }
        const size_t c = (size_t)(b - 1) * m->n3 + m->d.at(i, j, k);
        if (seen[c] || rst[c] == 0.0f) m->lists_unique = false;
        seen[c] = 1;
        rste[c] = rst[c];
      }
  if ((e = cudaMemcpy(m->resistive, rst.data(), rst.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(m->ctx, e, "resistive");
  if ((e = cudaMemcpy(m->rst_e, rste.data(), rste.size() * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_check(m->ctx, e, "rst_e");
  m->inner_set = true;
  return G3M3_OK;
}

int g3m3_model_init_steps(g3m3_model* m) {
  if (!m) return G3M3_ERR_ARG;
  for (int b = m->p.n_grids; b >= 1; b--) {
    m->t_old[b - 1] = 0.0;
    m->t_new[b - 1] = 0.0;
    int st = guard_stage(m, C, b, true, true);
    if (st) return st;
  }
  cudaError_t e = cudaMemcpyAsync(m->host_words, m->words, (8 + 5 * (size_t)G3M3_MAX_GRIDS) * sizeof(unsigned),
                                  cudaMemcpyDeviceToHost, S(m));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "init readback");
  if ((e = cudaStreamSynchronize(S(m))) != cudaSuccess) return cuda_check(m->ctx, e, "init sync");
  finish_steps(m, 1, m->p.n_grids);
  return G3M3_OK;
}

namespace {

int ensure_divb_boxes(g3m3_model* m) {
  if (m->cg_box) return G3M3_OK;
  const int ng = m->p.n_grids;
  cudaError_t e;
  if ((e = dev_alloc(m->ctx, (void**)&m->cg_box, ng * sizeof(CgState))) != cudaSuccess) return cuda_check(m->ctx, e, "div B state");
  if ((e = cudaMallocHost(&m->host_cg_box, ng * sizeof(CgState))) != cudaSuccess)
    return cuda_check(m->ctx, e, "div B state");
  if (ng > 1 && (e = dev_alloc(m->ctx, (void**)&m->cgvec_more, (size_t)(ng - 1) * 7 * m->n3 * sizeof(float))) != cudaSuccess)
    return cuda_check(m->ctx, e, "div B vectors");
  for (int b = 0; b < ng; b++) {
    if ((e = cudaStreamCreateWithFlags(&m->divb_stream[b], cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_check(m->ctx, e, "div B stream");
    if ((e = cudaEventCreateWithFlags(&m->divb_ev[b], cudaEventDisableTiming)) != cudaSuccess)
      return cuda_check(m->ctx, e, "div B event");
  }
  return G3M3_OK;
}

// divB_correct twice per box (3d_main.f90:1067-1096, 3363-3408), then the
// fine boxes' B copied onto the coarse ones.  A box's solves touch only its
// own B, so the boxes run side by side, each on its own stream with its own
// solver state and vectors; every solve is the same sequence of kernels as
// one run alone.  The pass is split into divb_begin (queue every box's
// first solve), divb_poll (advance every unfinished solve once; a box's
// second solve starts when its first has ended) and divb_end (join the box
// streams, flanks_synced and corer), so that an ensemble can keep the
// passes of all its members in flight together.
int divb_begin(g3m3_model* m) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  int st = ensure_divb_boxes(m);
  if (st) return st;
  G3M3_CUDA(m->ctx, cudaEventRecord(m->fork_ev, S(m)));
  for (int b = 1; b <= ng; b++) {
    CgRun& r = m->divb_run[b - 1];
    DivbArgs& a = r.a;
    a = DivbArgs{};
    a.bx = C(m, G3M3_F_BX, b); a.by = C(m, G3M3_F_BY, b); a.bz = C(m, G3M3_F_BZ, b);
    float* vec = b == 1 ? m->cgvec : m->cgvec_more + (size_t)(b - 2) * 7 * m->n3;
    const size_t n = m->n3;
    a.rhs = vec; a.x = vec + n; a.xs = vec + 2 * n; a.g = vec + 3 * n; a.h = vec + 4 * n;
    a.xi = vec + 5 * n; a.xj = vec + 6 * n;
    a.st = m->cg_box + (b - 1); a.d = m->d;
    a.rx = a.ry = a.rz = p.xspac[b - 1];
    r.host_st = m->host_cg_box + (b - 1);
    r.s = m->divb_stream[b - 1];
    r.graphs = &m->ctx->cg_graphs;
    m->divb_rep[b - 1] = 0;
    m->divb_fin[b - 1] = false;
    G3M3_CUDA(m->ctx, cudaStreamWaitEvent(r.s, m->fork_ev, 0));
  }
  m->divb_worst = G3M3_OK;
  for (int b = ng; b >= 1; b--) {
    const int h = m->cg_hint_box[b - 1] > 0 ? m->cg_hint_box[b - 1] : m->ctx->cg_hint;
    if ((st = cg_begin(m->ctx, m->divb_run[b - 1], p.divb_errlim, false, 1, h))) return st;
  }
  return G3M3_OK;
}

int divb_poll(g3m3_model* m, bool* all_done) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  int st;
  *all_done = true;
  for (int b = ng; b >= 1; b--) {
    if (m->divb_fin[b - 1]) continue;
    *all_done = false;
    CgRun& r = m->divb_run[b - 1];
    bool done = false;
    if ((st = cg_step(m->ctx, r, &done))) return st;
    if (!done) continue;
    const int iters = r.host_st->iters;
    if (r.status == CG_CONVERGED && iters > 0 && iters <= 4096) m->cg_hint_box[b - 1] = iters;
    if (r.status == CG_MAXIT) m->divb_worst = G3M3_ERR_NOCONV;
    divb_launch_apply(r.a, r.s);
    if (m->divb_rep[b - 1] == 0) {
      m->divb_rep[b - 1] = 1;
      const int h = m->cg_hint_box[b - 1] > 0 ? m->cg_hint_box[b - 1] : m->ctx->cg_hint;
      if ((st = cg_begin(m->ctx, r, p.divb_errlim, false, 1, h))) return st;
    } else {
      m->divb_fin[b - 1] = true;
    }
  }
  return G3M3_OK;
}

int divb_end(g3m3_model* m) {
  const g3m3_params& p = m->p;
  const int ng = p.n_grids;
  for (int b = 1; b <= ng; b++) {
    G3M3_CUDA(m->ctx, cudaEventRecord(m->divb_ev[b - 1], m->divb_run[b - 1].s));
    G3M3_CUDA(m->ctx, cudaStreamWaitEvent(S(m), m->divb_ev[b - 1], 0));
  }
  const int worst = m->divb_worst;
  if (worst) set_err(m->ctx, worst, "div B solver: too many iterations");
  for (int b = ng - 1; b >= 1; b--) {
    SyncedArgs a{};
    for (int q = 0; q < 3; q++) {
      a.fine[q] = C(m, G3M3_F_BX + q, b);
      a.coarse[q] = C(m, G3M3_F_BX + q, b + 1);
    }
    a.nf = 3;
    fill_synced_geometry(a, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax,
                         p.grd_zmin, p.grd_zmax);
    launch_flanks_synced(a, S(m));
  }
  for (int b = 1; b <= ng - 1; b++) corer_stage(m, b);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "divb_all");
  return worst;
}

}  // namespace

int g3m3_model_divb_all(g3m3_model* m) {
  if (!m) return G3M3_ERR_ARG;
  Range range("div B pass");
  if (m->tape) tape_divb(m);
  int st = divb_begin(m);
  for (bool done = false; !st && !done;) st = divb_poll(m, &done);
  return st ? st : divb_end(m);
}

namespace {

// One main step: plan, enqueue or replay, wait, finish (div B when due).
// The step graph of a planned main step: from the model's cache (keyed by
// buffer roles + actions), or captured on the model's stream -- scalar
// upload from the pinned table, the step, and the read-back of the recorded
// maxima -- and instantiated.
int step_graph(g3m3_model* m, const std::vector<Action>& acts, const std::string& key, cudaGraphExec_t* out) {
  auto found = m->graphs.find(key);
  if (found == m->graphs.end()) {
    cudaStream_t s = S(m);
    cudaError_t e;
    Roles saved = save_roles(m);
    cudaGraph_t g = nullptr;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return cuda_check(m->ctx, e, "begin capture");
    const int rc = step_enqueue(m, acts);
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    restore_roles(m, saved);   // capture did not run anything
    if (rc || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (rc) return rc;
      return cuda_check(m->ctx, e2, "graph capture");
    }
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_check(m->ctx, e, "graph instantiate");
    found = m->graphs.emplace(key, ex).first;
    m->kernel_nodes[key] = m->launches_in_step;
  }
  *out = found->second;
  return G3M3_OK;
}

int one_step(g3m3_model* m, int use_graph, std::vector<Action>& acts) {
  Range range("main step");
  cudaStream_t s = S(m);
  std::string key;
  int rc = step_plan(m, acts, key);
  if (rc) return rc;
  if (m->up_src) {   // the capture holds copies from this host buffer
    char buf[40];
    snprintf(buf, sizeof buf, "|up%p", (const void*)m->up_src);
    key += buf;
  }
  cudaError_t e;
  // a plan seen fewer than capture_after times runs host-launched: a
  // sub-cycling schedule that occurs once costs no capture
  if (use_graph && m->capture_after > 1 && !m->graphs.count(key) && ++m->plan_seen[key] < m->capture_after)
    use_graph = 0;
  if (use_graph) {
    cudaGraphExec_t ex = nullptr;
    if ((rc = step_graph(m, acts, key, &ex))) return rc;
    if ((e = cudaGraphLaunch(ex, s)) != cudaSuccess) return cuda_check(m->ctx, e, "graph launch");
    apply_role_swaps(m, acts);
    m->graph_launches += 1;
    m->kernels += m->kernel_nodes[key];
  } else {
    if ((rc = step_enqueue(m, acts))) return rc;
    m->kernels += m->launches_in_step;
  }
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_check(m->ctx, e, "main step");
  return step_finish(m);
}

int ensure_copy_stream(g3m3_model* m) {
  if (m->copy_stream) return G3M3_OK;
  G3M3_CUDA(m->ctx, cudaStreamCreateWithFlags(&m->copy_stream, cudaStreamNonBlocking));
  G3M3_CUDA(m->ctx, cudaEventCreateWithFlags(&m->up_fork, cudaEventDisableTiming));
  for (int b = 0; b < m->p.n_grids; b++)
    G3M3_CUDA(m->ctx, cudaEventCreateWithFlags(&m->up_ev[b], cudaEventDisableTiming));
  return G3M3_OK;
}

bool pinned(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

}  // namespace

int g3m3_model_run(g3m3_model* m, int nsteps, int use_graph) {
  if (!m || nsteps < 0) return G3M3_ERR_ARG;
  m->kernels = 0;
  m->graph_launches = 0;
  std::vector<Action> acts;
  for (int it = 0; it < nsteps; it++)
    if (int rc = one_step(m, use_graph, acts)) return rc;
  return G3M3_OK;
}

int g3m3_model_step_host(g3m3_model* m, const float* in, float* out, int use_graph) {
  if (!m || !in || !out) return G3M3_ERR_ARG;
  if (!finite_ok(m->ctx, in, (size_t)G3M3_NFIELDS * m->n4))
    return set_err(m->ctx, G3M3_ERR_NONFINITE, "host state holds NaN or Inf");
  m->kernels = 0;
  m->graph_launches = 0;
  if (!pinned(in)) {   // pageable input: plain upload, then the step
    int rc = g3m3_model_set_state(m, in);
    if (!rc) rc = g3m3_model_run(m, 1, use_graph);
    if (!rc) rc = g3m3_model_get_state(m, out);
    return rc;
  }
  int rc = ensure_copy_stream(m);
  if (rc) return rc;
  std::vector<Action> acts;
  m->up_src = in;
  rc = one_step(m, use_graph, acts);
  m->up_src = nullptr;
  if (rc) return rc;
  return g3m3_model_get_state(m, out);
}

int g3m3_model_time_kernel(g3m3_model* m, int kernel, int box, int reps, float* ms_per_launch, double* bytes) {
  if (!m || box < 1 || box > m->p.n_grids || reps < 1 || !ms_per_launch) return G3M3_ERR_ARG;
  const g3m3_params& p = m->p;
  const int b = box;
  const size_t n3 = m->n3;
  const size_t inner = (size_t)(m->d.nx - 2) * (m->d.ny - 2) * (m->d.nz - 2);
  const int slot = scal_slot(m, 0.01f);
  m->nscal = 0;
  if (slot < 0) return G3M3_ERR_STATE;
  cudaStream_t s = S(m);
  cudaError_t e = cudaMemcpyAsync(m->d_scal, m->h_scal, sizeof(float), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "time_kernel");
  double by = 0.0;
  auto launch = [&]() -> int {
    switch (kernel) {
      case 0: {  // corrector-form push of species q: src = cur, out = wrk
        PushIonArgs a{};
        for (int f = 0; f < 10; f++) { a.out[f] = W(m, f, b); a.old[f] = O(m, f, b); a.src[f] = C(m, f, b); }
        for (int q = 0; q < 3; q++) { a.bs[q] = m->bs[q]; a.efld[q] = m->efld[q]; a.tv[q] = m->tv[q]; }
        a.btot = m->btot; a.d = m->d;
        a.g.xmin = p.grd_xmin[b - 1]; a.g.ymin = p.grd_ymin[b - 1]; a.g.zmin = p.grd_zmin[b - 1];
        a.g.dx = (p.grd_xmax[b - 1] - p.grd_xmin[b - 1]) / (float)(m->d.nx - 1);
        a.g.dy = (p.grd_ymax[b - 1] - p.grd_ymin[b - 1]) / (float)(m->d.ny - 1);
        a.g.dz = (p.grd_zmax[b - 1] - p.grd_zmin[b - 1]) / (float)(m->d.nz - 1);
        a.rmass = p.rmassq; a.grav = p.grav; a.re_equiv = p.re_equiv; a.reynolds = p.reynolds;
        a.delt = sref(m, slot); a.boundary_from_old = 0; a.contracted = m->contracted;
        launch_push_ion(a, s);
        by = 160.0 * inner;     // 30 arrays read, 10 written per interior cell
        return 0;
      }
      case 1: {
        FcsArgs fa{};
        for (int q = 0; q < G3M3_NFIELDS; q++) {
          fa.px[q] = O(m, q, b); fa.old[q] = C(m, q, b); fa.wrk[q] = W(m, q, b);
          fa.chi[q] = q >= G3M3_F_BX ? p.diferg : p.difrho;
        }
        fa.nf = G3M3_NFIELDS; fa.d = m->d; fa.variant = m->fcs_variant;
        launch_fcsmooth(fa, s);
        by = 12.0 * G3M3_NFIELDS * n3;   // wrk, old read, result written, per field
        return 0;
      }
      case 2: {
        int st = guard_stage(m, W, b, true, false);
        by = (37.0 + 2.0) * 4.0 * n3;    // 30 species + epres + b + b0 read; btot, epres written
        return st;
      }
      case 3: {
        LapArgs la{};
        for (int f = 0; f < 10; f++) { la.in[f] = C(m, f, b); la.out[f] = W(m, f, b); la.chi[f] = 0.1f; }
        la.nf = 10;
        for (int q = 0; q < 3; q++) la.vp[q] = C(m, 1 + q, b);
        la.vrho = C(m, 0, b); la.vfloor = p.smallbit; la.d = m->d; la.delt = sref(m, slot);
        launch_lap(la, s);
        by = 80.0 * inner;
        return 0;
      }
      case 4: {
        if (b >= p.n_grids) return G3M3_ERR_ARG;
        FlanksArgs a{};
        for (int q = 0; q < G3M3_NFIELDS; q++) { a.target[q] = W(m, q, b); a.curc[q] = C(m, q, b + 1); a.oldc[q] = O(m, q, b + 1); }
        a.nf = G3M3_NFIELDS;
        fill_flanks_geometry(a, m->d.nx, m->d.ny, m->d.nz, b, p.grd_xmin, p.grd_xmax, p.grd_ymin, p.grd_ymax, p.grd_zmin, p.grd_zmax);
        a.t1 = sref(m, slot);
        launch_flanks(a, s);
        by = 8.0 * G3M3_NFIELDS * (double)shell_count(m->d, 2);   // shell read-modify-write
        return 0;
      }
      case 5: {
        CurrentArgs ca{};
        for (int q = 0; q < 3; q++) { ca.b[q] = C(m, G3M3_F_BX + q, b); ca.b0[q] = m->b0[q] + (size_t)(b - 1) * n3; ca.cur[q] = m->curr[q]; ca.bs[q] = m->bs[q]; }
        ca.btot = m->btot; ca.d = m->d;
        ca.rx = ca.ry = ca.rz = p.xspac[b - 1]; ca.smallbit = p.smallbit;
        launch_current(ca, s);
        by = 52.0 * n3;
        return 0;
      }
      case 6: {
        BandEArgs ba{};
        for (int q = 0; q < 3; q++) { ba.efld[q] = m->efld[q]; ba.bs[q] = m->bs[q]; ba.cur[q] = m->curr[q]; ba.ev[q] = m->ev[q]; ba.rho[q] = C(m, 10 * q, b); }
        ba.epres = C(m, G3M3_F_EPRES, b); ba.rst_e = nullptr; ba.d = m->d;
        ba.rmass[0] = p.rmassq; ba.rmass[1] = p.rmassh; ba.rmass[2] = p.rmasso;
        ba.reynolds = p.reynolds; ba.rx = ba.ry = ba.rz = p.xspac[b - 1];
        launch_bande(ba, s);
        by = 52.0 * n3;
        return 0;
      }
      default:
        return G3M3_ERR_ARG;
    }
  };
  int st = launch();   // warm-up
  if (st) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps && !st; r++) st = launch();
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "time_kernel");
  *ms_per_launch = ms / (float)reps;
  if (bytes) *bytes = by;
  return G3M3_OK;
}

int g3m3_model_write_fluid(g3m3_model* m, const char* path) {
  if (!m || !path) return G3M3_ERR_ARG;
  if (m->h_ij[0].empty()) return set_err(m->ctx, G3M3_ERR_STATE, "write_fluid: inner-boundary tables not set");
  const size_t n4 = m->n4;
  std::vector<float> state((size_t)G3M3_NFIELDS * n4), b0(3 * n4);
  int st = g3m3_model_get_state(m, state.data());
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(b0.data(), m->b0[0], 3 * n4 * sizeof(float), cudaMemcpyDeviceToHost, S(m));
  if (e == cudaSuccess) e = cudaStreamSynchronize(S(m));
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "write_fluid");
  const int mb = m->p.mbndry;
  std::vector<int> num[3];
  for (int l = 0; l < 3; l++) num[l].assign(m->num[l], m->num[l] + mb);
  return g3m3_fluid_write(m->ctx, path, &m->p, m->t, state.data(), b0.data(), m->h_parm[0].data(),
                          m->h_parm[1].data(), m->h_parm[2].data(), m->h_ij[2].data(), num[2].data(),
                          m->h_ij[1].data(), num[1].data(), m->h_ij[0].data(), num[0].data(), m->mlen[0], m->mlen[1],
                          m->mlen[2]);
}

int g3m3_model_read_fluid(g3m3_model* m, const char* path, int msrf, int mmid, int mzero) {
  if (!m || !path || msrf < 1 || mmid < 1 || mzero < 1) return G3M3_ERR_ARG;
  const size_t n4 = m->n4;
  const int mb = m->p.mbndry;
  std::vector<float> state((size_t)G3M3_NFIELDS * n4), b0(3 * n4);
  std::vector<float> parm[3] = {std::vector<float>((size_t)mb * 7 * msrf), std::vector<float>((size_t)mb * 7 * mmid),
                                std::vector<float>((size_t)mb * 7 * mzero)};
  std::vector<int> ij[3] = {std::vector<int>((size_t)mb * 3 * msrf), std::vector<int>((size_t)mb * 3 * mmid),
                            std::vector<int>((size_t)mb * 3 * mzero)};
  std::vector<int> num[3] = {std::vector<int>(mb), std::vector<int>(mb), std::vector<int>(mb)};
  double t = 0.0;
  int st = g3m3_fluid_read(m->ctx, path, &m->p, &t, state.data(), b0.data(), parm[0].data(), parm[1].data(),
                           parm[2].data(), ij[2].data(), num[2].data(), ij[1].data(), num[1].data(), ij[0].data(),
                           num[0].data(), msrf, mmid, mzero);
  if (st) return st;
  if ((st = g3m3_model_set_state(m, state.data()))) return st;
  // the wrk copy starts as the state (wrkepres is read before it is written)
  for (int q = 0; q < G3M3_NFIELDS; q++)
    if ((st = g3m3_model_set_field(m, 2, q, state.data() + (size_t)q * n4))) return st;
  if ((st = g3m3_model_set_b0(m, b0.data(), b0.data() + n4, b0.data() + 2 * n4))) return st;
  // the resistivity is not part of the file: keep the model's
  std::vector<float> rst((size_t)mb * m->n3);
  cudaError_t e = cudaMemcpy(rst.data(), m->resistive, rst.size() * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "read_fluid");
  if ((st = g3m3_model_set_inner(m, rst.data(), ij[0].data(), num[0].data(), parm[0].data(), msrf, ij[1].data(),
                                 num[1].data(), parm[1].data(), mmid, ij[2].data(), num[2].data(), parm[2].data(),
                                 mzero)))
    return st;
  m->t = t;
  return G3M3_OK;
}

int g3m3_model_graphing(g3m3_model* m, int box, int plane, int index, float* out) {
  if (!m || !out || box < 1 || box > m->p.n_grids || plane < 0 || plane > 2) return G3M3_ERR_ARG;
  const Dims d = m->d;
  const int lim = plane == 0 ? d.nz : (plane == 1 ? d.ny : d.nx);
  if (index < 1 || index > lim) return set_err(m->ctx, G3M3_ERR_ARG, "graphing: plane index %d outside 1..%d", index, lim);
  const int na = plane == 0 ? d.ny : d.nz, nb = plane == 2 ? d.ny : d.nx;
  const size_t per = (size_t)na * nb;
  float* dout = nullptr;
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&dout, 32 * per * sizeof(float)));
  // J, total B, |B|, E of the box as the step computes them (calcur, fnd_evel, BandE)
  fields_stage(m, C, box);
  auto cut = [&](std::initializer_list<const float*> src, int q0) {
    CutArgs a{};
    int n = 0;
    for (const float* p : src) a.src[n++] = p;
    a.nq = n; a.q0 = q0; a.plane = plane; a.index = index; a.d = d; a.out = dout;
    launch_cut(a, S(m));
  };
  cut({m->bs[0], m->bs[1], m->bs[2], m->btot, m->efld[0], m->efld[1], m->efld[2], m->curr[0], m->curr[1],
       m->curr[2]}, 0);
  // per species: velocity with the density floor, pressure parallel /
  // perpendicular / cross (fnd_pres), density
  for (int sp = 0; sp < 3; sp++) {
    const float* pm[3] = {C(m, 10 * sp + 1, box), C(m, 10 * sp + 2, box), C(m, 10 * sp + 3, box)};
    float* v[3] = {m->vt[0], m->vt[1], m->vt[2]};
    launch_velocity_floor(C(m, 10 * sp, box), pm, v, m->p.smallbit, m->n3, S(m));
    const float* pr[3] = {C(m, 10 * sp + 4, box), C(m, 10 * sp + 5, box), C(m, 10 * sp + 6, box)};
    const float* vv[3] = {m->vt[0], m->vt[1], m->vt[2]};
    const float* bt[3] = {m->bs[0], m->bs[1], m->bs[2]};
    launch_fnd_pres(pr, m->ev[0], m->ev[1], m->ev[2], vv, bt, d, S(m));
    cut({m->vt[0], m->vt[1], m->vt[2], m->ev[0], m->ev[1], m->ev[2], C(m, 10 * sp, box)}, 10 + 7 * sp);
  }
  cut({C(m, G3M3_F_EPRES, box)}, 31);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 32 * per * sizeof(float), cudaMemcpyDeviceToHost, S(m));
  if (e == cudaSuccess) e = cudaStreamSynchronize(S(m));
  cudaFree(dout);
  return e == cudaSuccess ? G3M3_OK : cuda_check(m->ctx, e, "graphing");
}

int g3m3_model_init_state(g3m3_model* m, float alf_inner, unsigned long long seed, float noise, float iono_lo,
                          float iono_hi) {
  if (!m || noise < 0.0f || !(iono_lo > 0.0f) || iono_hi < iono_lo) return G3M3_ERR_ARG;
  const g3m3_params& p = m->p;
  const int nx = p.nx, ny = p.ny, nz = p.nz, mb = p.mbndry;
  const double r_inner = p.r_inner;
  const double zero_b = r_inner - 1.5, mid_b = r_inner - 0.5, srf_b = r_inner + 0.6;
  const double b0c = (double)alf_inner * std::sqrt((double)p.erho) * (r_inner * r_inner * r_inner);
  const double xdip = 0.00001;
  // per-cell fields of every box on the device
  for (int b = 1; b <= p.n_grids; b++) {
    InitArgs a{};
    for (int q = 0; q < G3M3_NFIELDS; q++) a.f[q] = C(m, q, b);
    for (int q = 0; q < 3; q++) a.b0[q] = m->b0[q] + (size_t)(b - 1) * m->n3;
    a.d = m->d; a.box = b;
    a.xmin = p.grd_xmin[b - 1]; a.ymin = p.grd_ymin[b - 1]; a.zmin = p.grd_zmin[b - 1];
    a.dx = ((double)p.grd_xmax[b - 1] - p.grd_xmin[b - 1]) / (nx - 1.0);
    a.dy = ((double)p.grd_ymax[b - 1] - p.grd_ymin[b - 1]) / (ny - 1.0);
    a.dz = ((double)p.grd_zmax[b - 1] - p.grd_zmin[b - 1]) / (nz - 1.0);
    a.b0c = b0c; a.zero_b = zero_b; a.re_equiv = p.re_equiv; a.r_rot = p.r_rot; a.v_rot = p.v_rot;
    a.r_inner = r_inner; a.alpha_e = p.alpha_e; a.erho = p.erho; a.d_min = 0.01; a.cs_inner = 0.0163;
    a.ti_te = p.ti_te; a.gamma = p.gamma; a.spress = p.spress; a.srho = p.srho;
    a.spx = p.spx; a.spy = p.spy; a.spz = p.spz; a.rho_frac = p.rho_frac;
    a.rmass[0] = p.rmassq; a.rmass[1] = p.rmassh; a.rmass[2] = p.rmasso;
    a.noise = noise; a.seed = seed;
    launch_init(a, S(m));
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "init_state");
  // the wrk copy starts as the state (wrkepres is read before it is written)
  for (int q = 0; q < G3M3_NFIELDS; q++)
    for (int b = 1; b <= p.n_grids; b++)
      if ((e = cudaMemcpyAsync(W(m, q, b), C(m, q, b), m->n3 * sizeof(float), cudaMemcpyDeviceToDevice, S(m))) !=
          cudaSuccess)
        return cuda_check(m->ctx, e, "init_state");
  // inner-boundary lists of boxes <= mbndry (3d_main.f90:1374-1452), in the
  // reference's loop order, with the cell's density and pressure values
  const int parm_fields[7] = {0, 10, 20, 4, 14, 24, G3M3_F_EPRES};
  std::vector<int> ij[3];
  std::vector<float> parm[3];
  std::vector<int> nums[3];
  std::vector<std::vector<std::array<int, 3>>> cells(3 * mb);
  std::vector<std::vector<std::array<float, 7>>> vals(3 * mb);
  std::vector<float> host((size_t)7 * m->n3);
  for (int b = 1; b <= mb; b++) {
    for (int q = 0; q < 7; q++)
      if ((e = cudaMemcpyAsync(host.data() + (size_t)q * m->n3, C(m, parm_fields[q], b), m->n3 * sizeof(float),
                               cudaMemcpyDeviceToHost, S(m))) != cudaSuccess)
        return cuda_check(m->ctx, e, "init_state");
    if ((e = cudaStreamSynchronize(S(m))) != cudaSuccess) return cuda_check(m->ctx, e, "init_state");
    const double dx = ((double)p.grd_xmax[b - 1] - p.grd_xmin[b - 1]) / (nx - 1.0);
    const double dy = ((double)p.grd_ymax[b - 1] - p.grd_ymin[b - 1]) / (ny - 1.0);
    const double dz = ((double)p.grd_zmax[b - 1] - p.grd_zmin[b - 1]) / (nz - 1.0);
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
          const double ax = (double)p.grd_xmin[b - 1] + dx * i - xdip;
          const double ay = (double)p.grd_ymin[b - 1] + dy * j;
          const double az = (double)p.grd_zmin[b - 1] + dz * k;
          const double ar = std::sqrt(ax * ax + ay * ay + az * az);
          if (!(ar <= srf_b)) continue;
          const int l = ar < zero_b ? 2 : (ar < mid_b ? 1 : 0);   // 0 srf, 1 mid, 2 zero
          const size_t c = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
          std::array<float, 7> v;
          for (int q = 0; q < 7; q++) v[q] = host[(size_t)q * m->n3 + c];
          cells[3 * (b - 1) + l].push_back({i + 1, j + 1, k + 1});
          vals[3 * (b - 1) + l].push_back(v);
        }
  }
  // ionospheric inflow densities, log-uniform per list entry
  unsigned long long rs = seed ^ 0x5851f42d4c957f2dull;
  auto uni = [&]() {
    rs += 0x9e3779b97f4a7c15ull;
    unsigned long long z = rs;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return (double)((z ^ (z >> 31)) >> 11) * 0x1p-53;
  };
  for (int l = 0; l < 3; l++)
    for (int b = 1; b <= mb; b++)
      for (auto& v : vals[3 * (b - 1) + l]) {
        const double f = iono_hi > iono_lo
                             ? std::exp(std::log((double)iono_lo) + uni() * (std::log((double)iono_hi) - std::log((double)iono_lo)))
                             : 1.0;
        for (int q = 0; q < 3; q++) v[q] = (float)(v[q] * f);
      }
  int ml[3];
  for (int l = 0; l < 3; l++) {
    ml[l] = 1;
    for (int b = 1; b <= mb; b++) ml[l] = std::max(ml[l], (int)cells[3 * (b - 1) + l].size());
    ij[l].assign((size_t)mb * 3 * ml[l], 0);
    parm[l].assign((size_t)mb * 7 * ml[l], 0.0f);
    nums[l].assign(mb, 0);
    for (int b = 1; b <= mb; b++) {
      const auto& cl = cells[3 * (b - 1) + l];
      const auto& vl = vals[3 * (b - 1) + l];
      nums[l][b - 1] = (int)cl.size();
      for (size_t n = 0; n < cl.size(); n++) {
        for (int q = 0; q < 3; q++) ij[l][(b - 1) + (size_t)mb * (q + 3 * n)] = cl[n][q];
        for (int q = 0; q < 7; q++) parm[l][(b - 1) + (size_t)mb * (q + 7 * n)] = vl[n][q];
      }
    }
  }
  // set_resist with b0 = 1 (sub_set_resist.f90:10-63)
  std::vector<float> rst((size_t)mb * m->n3, 0.0f);
  const float rval[3] = {0.125f / p.resist, 0.5f / p.resist, 1.0f / p.resist};
  for (int l : {2, 1, 0})
    for (int b = 1; b <= mb; b++)
      for (const auto& c3 : cells[3 * (b - 1) + l])
        rst[(size_t)(b - 1) * m->n3 + (size_t)(c3[0] - 1) + (size_t)nx * ((size_t)(c3[1] - 1) + (size_t)ny * (c3[2] - 1))] =
            rval[l];
  return g3m3_model_set_inner(m, rst.data(), ij[0].data(), nums[0].data(), parm[0].data(), ml[0], ij[1].data(),
                              nums[1].data(), parm[1].data(), ml[1], ij[2].data(), nums[2].data(), parm[2].data(),
                              ml[2]);
}

int g3m3_model_record_craft(g3m3_model* m, int ncraft, const int* npts, const float* traj, int nf,
                            const int* fields, int capacity) {
  if (!m || ncraft < 0 || ncraft > 128 || nf < 0 || nf > 8 || capacity < 0) return G3M3_ERR_ARG;
  if (capacity > 0 && (ncraft < 1 || nf < 1 || !npts || !traj || !fields)) return G3M3_ERR_ARG;
  cudaStreamSynchronize(S(m));
  float** bufs[3] = {&m->craft_traj, &m->craft_out, nullptr};
  for (int q = 0; q < 2; q++)
    if (*bufs[q]) { cudaFree(*bufs[q]); *bufs[q] = nullptr; }
  if (m->craft_start) { cudaFree(m->craft_start); m->craft_start = nullptr; }
  if (m->craft_count) { cudaFree(m->craft_count); m->craft_count = nullptr; }
  m->craft_cap = 0;
  m->ncraft = 0;
  // the recording launch changes the step's launch sequence
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  m->kernel_nodes.clear();
  if (capacity == 0) return G3M3_OK;
  std::vector<int> start(ncraft + 1, 0);
  for (int c = 0; c < ncraft; c++) {
    if (npts[c] < 1) return set_err(m->ctx, G3M3_ERR_ARG, "craft %d has no trajectory samples", c);
    start[c + 1] = start[c] + npts[c];
  }
  for (int f = 0; f < nf; f++) {
    if (fields[f] < 0 || fields[f] >= G3M3_NFIELDS) return set_err(m->ctx, G3M3_ERR_ARG, "bad field index");
    m->craft_fields[f] = fields[f];
  }
  const size_t nrec = (size_t)capacity * ncraft * (4 + nf);
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->craft_traj, (size_t)4 * start[ncraft] * sizeof(float)));
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->craft_start, (ncraft + 1) * sizeof(int)));
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->craft_out, nrec * sizeof(float)));
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->craft_count, sizeof(unsigned)));
  G3M3_CUDA(m->ctx, cudaMemcpy(m->craft_traj, traj, (size_t)4 * start[ncraft] * sizeof(float), cudaMemcpyDefault));
  G3M3_CUDA(m->ctx, cudaMemcpy(m->craft_start, start.data(), (ncraft + 1) * sizeof(int), cudaMemcpyHostToDevice));
  G3M3_CUDA(m->ctx, cudaMemset(m->craft_count, 0, sizeof(unsigned)));
  m->ncraft = ncraft;
  m->craft_nf = nf;
  m->craft_cap = capacity;
  return G3M3_OK;
}

int g3m3_model_craft_records(g3m3_model* m, float* out, int* nsteps) {
  if (!m) return G3M3_ERR_ARG;
  unsigned n = 0;
  if (m->craft_cap > 0) {
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(&n, m->craft_count, sizeof(unsigned), cudaMemcpyDeviceToHost, S(m)));
    G3M3_CUDA(m->ctx, cudaStreamSynchronize(S(m)));
    if (n > (unsigned)m->craft_cap) n = (unsigned)m->craft_cap;
    if (out && n > 0) {
      G3M3_CUDA(m->ctx, cudaMemcpyAsync(out, m->craft_out, (size_t)n * m->ncraft * (4 + m->craft_nf) * sizeof(float),
                                        cudaMemcpyDeviceToHost, S(m)));
      G3M3_CUDA(m->ctx, cudaStreamSynchronize(S(m)));
    }
  }
  if (nsteps) *nsteps = (int)n;
  return G3M3_OK;
}

int g3m3_model_record_fluxes(g3m3_model* m, const float* scale, int capacity) {
  if (!m || capacity < 0 || (capacity > 0 && !scale)) return G3M3_ERR_ARG;
  cudaStreamSynchronize(S(m));
  if (m->flux_hist) cudaFree(m->flux_hist);
  if (m->flux_count) cudaFree(m->flux_count);
  m->flux_hist = nullptr;
  m->flux_count = nullptr;
  m->flux_cap = 0;
  // the recording launches change the step's launch sequence
  for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
  m->graphs.clear();
  m->kernel_nodes.clear();
  if (capacity == 0) return G3M3_OK;
  const size_t n = (size_t)capacity * m->p.n_grids * 6;
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->flux_hist, n * sizeof(float)));
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&m->flux_count, sizeof(unsigned)));
  G3M3_CUDA(m->ctx, cudaMemsetAsync(m->flux_count, 0, sizeof(unsigned), S(m)));
  G3M3_CUDA(m->ctx, cudaMemsetAsync(m->flux_hist, 0, n * sizeof(float), S(m)));
  std::memcpy(m->flux_scale, scale, m->p.n_grids * sizeof(float));
  m->flux_cap = capacity;
  return G3M3_OK;
}

int g3m3_model_fluxes(g3m3_model* m, float* out, int* nsteps) {
  if (!m) return G3M3_ERR_ARG;
  unsigned n = 0;
  if (m->flux_cap > 0) {
    G3M3_CUDA(m->ctx, cudaMemcpyAsync(&n, m->flux_count, sizeof(unsigned), cudaMemcpyDeviceToHost, S(m)));
    G3M3_CUDA(m->ctx, cudaStreamSynchronize(S(m)));
    if (n > (unsigned)m->flux_cap) n = (unsigned)m->flux_cap;
    if (out && n > 0) {
      G3M3_CUDA(m->ctx, cudaMemcpyAsync(out, m->flux_hist, (size_t)n * m->p.n_grids * 6 * sizeof(float),
                                        cudaMemcpyDeviceToHost, S(m)));
      G3M3_CUDA(m->ctx, cudaStreamSynchronize(S(m)));
    }
  }
  if (nsteps) *nsteps = (int)n;
  return G3M3_OK;
}

int g3m3_model_set_contracted(g3m3_model* m, int on) {
  if (!m) return G3M3_ERR_ARG;
  if (m->contracted != (on != 0)) {
    for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);   // graphs hold the other kernels
    m->graphs.clear();
    m->kernel_nodes.clear();
    m->contracted = on != 0;
  }
  return G3M3_OK;
}

int g3m3_model_set_variant(g3m3_model* m, int kernel, int variant) {
  if (!m || kernel != 1 || variant < 0 || variant >= G3M3_FCS_VARIANTS) return G3M3_ERR_ARG;
  G3M3_CUDA(m->ctx, prepare_fcsmooth());
  if (m->fcs_variant != variant) {
    // captured graphs hold the old launch shape
    for (auto& kv : m->graphs) cudaGraphExecDestroy(kv.second);
    m->graphs.clear();
    m->kernel_nodes.clear();
    m->fcs_variant = variant;
  }
  return G3M3_OK;
}

int g3m3_model_autotune(g3m3_model* m, int* fcs_variant) {
  if (!m) return G3M3_ERR_ARG;
  cudaStream_t s = S(m);
  const size_t n3 = m->n3;
  // scratch copies of box 1's current, old and wrk fields: timing runs on
  // realistic values without touching the state
  float* tmp = nullptr;
  G3M3_CUDA(m->ctx, dev_alloc(m->ctx, (void**)&tmp, 3 * (size_t)G3M3_NFIELDS * n3 * sizeof(float)));
  FcsArgs fa{};
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < G3M3_NFIELDS && e == cudaSuccess; q++) {
    float* px = tmp + (size_t)q * n3;
    float* od = tmp + (size_t)(G3M3_NFIELDS + q) * n3;
    float* wk = tmp + (size_t)(2 * G3M3_NFIELDS + q) * n3;
    e = cudaMemcpyAsync(od, O(m, q, 1), n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(wk, C(m, q, 1), n3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    fa.px[q] = px; fa.old[q] = od; fa.wrk[q] = wk;
    fa.chi[q] = q >= G3M3_F_BX ? m->p.diferg : m->p.difrho;
  }
  fa.nf = G3M3_NFIELDS; fa.d = m->d;
  if (e == cudaSuccess) e = prepare_fcsmooth();
  float best_ms = 0.0f;
  int best = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int v = 0; v < G3M3_FCS_VARIANTS && e == cudaSuccess; v++) {
    fa.variant = v;
    launch_fcsmooth(fa, s);   // warm-up
    cudaEventRecord(e0, s);
    for (int r = 0; r < 5; r++) launch_fcsmooth(fa, s);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && (v == 0 || ms < best_ms)) { best_ms = ms; best = v; }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(tmp);
  if (e != cudaSuccess) return cuda_check(m->ctx, e, "autotune");
  if (fcs_variant) *fcs_variant = best;
  return g3m3_model_set_variant(m, 1, best);
}

int g3m3_model_times(g3m3_model* m, double* t, double* t_stepnew, int64_t* cell_updates) {
  if (!m) return G3M3_ERR_ARG;
  if (t) *t = m->t;
  if (t_stepnew) std::memcpy(t_stepnew, m->t_stepnew, m->p.n_grids * sizeof(double));
  if (cell_updates) *cell_updates = m->cell_updates;
  return G3M3_OK;
}

int g3m3_model_set_capture_after(g3m3_model* m, int n) {
  if (!m || n < 1) return G3M3_ERR_ARG;
  m->capture_after = n;
  m->plan_seen.clear();
  return G3M3_OK;
}

int g3m3_model_get_clock(g3m3_model* m, double* t, int* nsteps_done) {
  if (!m) return G3M3_ERR_ARG;
  if (t) *t = m->t;
  if (nsteps_done) *nsteps_done = m->nsteps_done;
  return G3M3_OK;
}

int g3m3_model_set_clock(g3m3_model* m, double t, int nsteps_done) {
  if (!m || nsteps_done < 0) return G3M3_ERR_ARG;
  m->t = t;
  m->nsteps_done = nsteps_done;
  return G3M3_OK;
}

int g3m3_model_stats(g3m3_model* m, int64_t* kernels, int64_t* graphs) {
  if (!m) return G3M3_ERR_ARG;
  if (kernels) *kernels = m->kernels;
  if (graphs) *graphs = m->graph_launches;
  return G3M3_OK;
}

// --------------------------------------------------------------------------
// Ensembles: independent states (e.g. one per upstream condition, boxes of
// different sizes) advanced together.  Each member is a model with its own
// stream.  In graph mode one main step of every member is captured into a
// single CUDA graph -- fork from the ensemble's stream, each member's step on
// its own stream, join -- so the members' kernels overlap on the GPU; the
// graph is cached by the members' combined schedule key.  In plain mode the
// members step one after another from the host loop.
// --------------------------------------------------------------------------
}  // extern "C"

struct g3m3_ensemble {
  g3m3_ctx* ctx = nullptr;
  std::vector<g3m3_model*> members;
  std::vector<cudaEvent_t> done;
  cudaEvent_t fork = nullptr;
  std::map<std::string, cudaGraphExec_t> graphs;
  std::map<std::string, int64_t> kernel_nodes;
  int64_t kernels = 0, graph_launches = 0;
};

extern "C" {

int g3m3_ensemble_destroy(g3m3_ensemble* e) {
  if (!e) return G3M3_ERR_ARG;
  cudaStreamSynchronize(e->ctx->stream);
  for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
  for (g3m3_model* m : e->members) g3m3_model_destroy(m);
  for (cudaEvent_t ev : e->done) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  delete e;
  return G3M3_OK;
}

int g3m3_ensemble_create(g3m3_ctx* ctx, int n, const g3m3_params* params, g3m3_ensemble** out) {
  if (!ctx || !params || !out || n < 1) return G3M3_ERR_ARG;
  *out = nullptr;
  g3m3_ensemble* e = new g3m3_ensemble();
  e->ctx = ctx;
  cudaError_t ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  for (int i = 0; i < n && ce == cudaSuccess; i++) {
    g3m3_model* m = nullptr;
    cudaStream_t st = nullptr;
    if ((ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) break;
    const int rc = g3m3_model_create(ctx, &params[i], &m);
    if (rc) {
      cudaStreamDestroy(st);
      g3m3_ensemble_destroy(e);
      return rc;
    }
    // the model's set-up work ran on the context's stream
    cudaStreamSynchronize(ctx->stream);
    m->stream = st;
    m->own_stream = true;
    e->members.push_back(m);
    cudaEvent_t ev = nullptr;
    if ((ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) break;
    e->done.push_back(ev);
  }
  if (ce != cudaSuccess) {
    const int rc = cuda_check(ctx, ce, "ensemble create");
    g3m3_ensemble_destroy(e);
    return rc;
  }
  *out = e;
  return G3M3_OK;
}

int g3m3_ensemble_member(g3m3_ensemble* e, int i, g3m3_model** out) {
  if (!e || !out || i < 0 || i >= (int)e->members.size()) return G3M3_ERR_ARG;
  *out = e->members[i];
  return G3M3_OK;
}

void* g3m3_ensemble_stream(g3m3_ensemble* e) { return e ? (void*)e->ctx->stream : nullptr; }

namespace {

// The members' step ends; the div B passes that are due run together, every
// member's boxes solving side by side (their results are those of each
// member alone).
int finish_members(g3m3_ensemble* e) {
  const size_t nm = e->members.size();
  std::vector<char> due(nm, 0);
  bool any = false;
  for (size_t i = 0; i < nm; i++) {
    bool d = false;
    if (int rc = step_finish(e->members[i], &d)) return rc;
    due[i] = d;
    any = any || d;
  }
  if (!any) return G3M3_OK;
  for (size_t i = 0; i < nm; i++)
    if (due[i])
      if (int rc = divb_begin(e->members[i])) return rc;
  for (bool busy = true; busy;) {
    busy = false;
    for (size_t i = 0; i < nm; i++) {
      if (!due[i]) continue;
      bool done = false;
      if (int rc = divb_poll(e->members[i], &done)) return rc;
      if (done) due[i] = 2;   // polled to the end: joined below
      else busy = true;
    }
    for (size_t i = 0; i < nm; i++)
      if (due[i] == 2) {
        g3m3_model* m = e->members[i];
        const int rc = divb_end(m);
        if (rc && rc != G3M3_ERR_NOCONV) return rc;
        cudaError_t ce = cudaStreamSynchronize(S(m));
        if (ce != cudaSuccess) return cuda_check(e->ctx, ce, "divb");
        due[i] = 0;
      }
  }
  return G3M3_OK;
}

}  // namespace

int g3m3_ensemble_run(g3m3_ensemble* e, int nsteps, int use_graph) {
  if (!e || nsteps < 0 || use_graph < 0 || use_graph > 3) return G3M3_ERR_ARG;
  // 0: members one after another; 1: one graph per main step; 2: every
  // member launched from the host on its own stream, all at once; 3: every
  // member's own step graph launched on its own stream, all at once
  const bool member_graphs = use_graph == 3;
  const bool concurrent = use_graph == 2;
  if (use_graph == 2 || use_graph == 3) use_graph = 0;
  const size_t nm = e->members.size();
  cudaStream_t origin = e->ctx->stream;
  e->kernels = 0;
  e->graph_launches = 0;
  std::vector<std::vector<Action>> acts(nm);
  std::vector<std::string> keys(nm);
  cudaError_t ce;
  for (int it = 0; it < nsteps; it++) {
    std::string key;
    for (size_t i = 0; i < nm; i++) {
      const int rc = step_plan(e->members[i], acts[i], keys[i]);
      if (rc) return rc;
      key += keys[i];
      key += '|';
    }
    if (member_graphs) {
      // find or capture every member's graph first (captures are isolated),
      // then launch them all between the fork and join events
      std::vector<cudaGraphExec_t> ex(nm);
      for (size_t i = 0; i < nm; i++)
        if (int rc = step_graph(e->members[i], acts[i], keys[i], &ex[i])) return rc;
      if ((ce = cudaEventRecord(e->fork, origin)) != cudaSuccess) return cuda_check(e->ctx, ce, "fork");
      for (size_t i = 0; i < nm; i++) {
        g3m3_model* m = e->members[i];
        if ((ce = cudaStreamWaitEvent(S(m), e->fork, 0)) != cudaSuccess) return cuda_check(e->ctx, ce, "fork");
        if ((ce = cudaGraphLaunch(ex[i], S(m))) != cudaSuccess) return cuda_check(e->ctx, ce, "graph launch");
        apply_role_swaps(m, acts[i]);
        e->kernels += m->kernel_nodes[keys[i]];
        e->graph_launches += 1;
        if ((ce = cudaEventRecord(e->done[i], S(m))) != cudaSuccess) return cuda_check(e->ctx, ce, "join");
        if ((ce = cudaStreamWaitEvent(origin, e->done[i], 0)) != cudaSuccess) return cuda_check(e->ctx, ce, "join");
      }
      if ((ce = cudaStreamSynchronize(origin)) != cudaSuccess) return cuda_check(e->ctx, ce, "ensemble step");
      if (int rc = finish_members(e)) return rc;
      continue;
    }
    // every member's step is ordered after earlier work on the ensemble's
    // stream and the ensemble's stream after every member's step, so events
    // recorded there bracket the whole step in both modes
    // In the one-graph form the members' steps form kGraphChains chains of
    // members, one after another within a chain, and each member's stages
    // run on its own stream only (its side streams folded in): the graph
    // executor overlapped 16 member branches of four streams each far worse
    // (542 M cell-updates/s on the 16-member bench ensemble) than 2 chains
    // of single-stream members (765 M; 4 chains 706 M, 8 659 M, 1 649 M).
    constexpr size_t kGraphChains = 2;
    auto fork_join = [&](bool capture_mode) -> int {
      int64_t nk = 0;
      if ((ce = cudaEventRecord(e->fork, origin)) != cudaSuccess) return cuda_check(e->ctx, ce, "fork");
      for (size_t i = 0; i < nm; i++) {
        g3m3_model* m = e->members[i];
        const cudaEvent_t after = (capture_mode && i >= kGraphChains) ? e->done[i - kGraphChains] : e->fork;
        if ((ce = cudaStreamWaitEvent(S(m), after, 0)) != cudaSuccess) return cuda_check(e->ctx, ce, "fork");
        const int rc = step_enqueue(m, acts[i]);
        if (rc) return rc;
        nk += m->launches_in_step;
        if ((ce = cudaEventRecord(e->done[i], S(m))) != cudaSuccess) return cuda_check(e->ctx, ce, "join");
        if ((ce = cudaStreamWaitEvent(origin, e->done[i], 0)) != cudaSuccess) return cuda_check(e->ctx, ce, "join");
        if (!capture_mode && !concurrent) {
          // plain mode: one member at a time, launched from the host loop
          if ((ce = cudaStreamSynchronize(S(m))) != cudaSuccess) return cuda_check(e->ctx, ce, "member step");
        }
      }
      e->kernels += capture_mode ? 0 : nk;
      if (capture_mode) e->kernel_nodes[key] = nk;
      return G3M3_OK;
    };
    if (use_graph) {
      auto found = e->graphs.find(key);
      if (found == e->graphs.end()) {
        std::vector<Roles> saved(nm);
        for (size_t i = 0; i < nm; i++) saved[i] = save_roles(e->members[i]);
        cudaGraph_t g = nullptr;
        // side streams folded into each member's stream for the capture
        std::vector<std::array<cudaStream_t, 3>> aux_saved(nm);
        for (size_t i = 0; i < nm; i++) {
          g3m3_model* mm = e->members[i];
          for (int q = 0; q < 3; q++) {
            aux_saved[i][q] = mm->aux[q];
            mm->aux[q] = S(mm);
          }
        }
        if ((ce = cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
          for (size_t i = 0; i < nm; i++)
            for (int q = 0; q < 3; q++) e->members[i]->aux[q] = aux_saved[i][q];
          return cuda_check(e->ctx, ce, "begin capture");
        }
        const int rc = fork_join(true);
        const cudaError_t e2 = cudaStreamEndCapture(origin, &g);
        for (size_t i = 0; i < nm; i++)
          for (int q = 0; q < 3; q++) e->members[i]->aux[q] = aux_saved[i][q];
        for (size_t i = 0; i < nm; i++) restore_roles(e->members[i], saved[i]);
        if (rc || e2 != cudaSuccess) {
          if (g) cudaGraphDestroy(g);
          if (rc) return rc;
          return cuda_check(e->ctx, e2, "graph capture");
        }
        cudaGraphExec_t ex = nullptr;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_check(e->ctx, ce, "graph instantiate");
        found = e->graphs.emplace(key, ex).first;
      }
      if ((ce = cudaGraphLaunch(found->second, origin)) != cudaSuccess) return cuda_check(e->ctx, ce, "graph launch");
      for (size_t i = 0; i < nm; i++) apply_role_swaps(e->members[i], acts[i]);
      e->graph_launches += 1;
      e->kernels += e->kernel_nodes[key];
    } else {
      const int rc = fork_join(false);
      if (rc) return rc;
    }
    if ((ce = cudaStreamSynchronize(origin)) != cudaSuccess) return cuda_check(e->ctx, ce, "ensemble step");
    if (int rc = finish_members(e)) return rc;
  }
  return G3M3_OK;
}

int g3m3_ensemble_stats(g3m3_ensemble* e, int64_t* kernels, int64_t* graphs, int64_t* cell_updates) {
  if (!e) return G3M3_ERR_ARG;
  if (kernels) *kernels = e->kernels;
  if (graphs) *graphs = e->graph_launches;
  if (cell_updates) {
    int64_t cu = 0;
    for (g3m3_model* m : e->members) cu += m->cell_updates;
    *cell_updates = cu;
  }
  return G3M3_OK;
}

}  // extern "C"
