// model.cuh -- the step engine's model (g3m3_model_*): a whole multi-box
// state on the device, its scratch, schedule bookkeeping and graph cache.
// Shared by the engine (engine.cu) and its adjoint (adjoint.cu).
#pragma once

#include <map>
#include <string>
#include <vector>

#include "bndry.cuh"
#include "ctx.cuh"

namespace g3m3 {
struct Tape;   // adjoint.cu: snapshots of the recorded main steps

// Where the engine hands a recording to the tape (adjoint.cu).  Each point
// names the state it snapshots: the predictor's, corrector's, Lapidus' and
// flux correction's result after its boundaries (before the guards), and
// after its guards.
enum TapePoint {
  TP_PRED_BNDRY = 0, TP_PRED_GUARD, TP_CORR_BNDRY, TP_CORR_GUARD, TP_LAP_BNDRY, TP_LAP_GUARD, TP_FCS_BNDRY,
  TP_NPOINTS
};
}  // namespace g3m3

struct g3m3_model {
  g3m3_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;     // the context's stream, or the member's own in an ensemble
  bool own_stream = false;
  cudaStream_t aux[3] = {};          // side streams for independent kernels of a stage
  cudaEvent_t fork_ev = nullptr, join_ev[3] = {};
  g3m3_params p{};
  g3m3::Dims d{};
  size_t n3 = 0, n4 = 0;
  float* mem = nullptr;              // one allocation for every array below
  float* buf[3][G3M3_NFIELDS] = {};  // three full (nx,ny,nz,n_grids) copies per field
  int role_cur[G3M3_MAX_GRIDS] = {}, role_old[G3M3_MAX_GRIDS] = {};
  float* b0[3] = {};
  float* resistive = nullptr;
  float* rst_e = nullptr;            // BandE's resistive coefficient per cell (0: none)
  bool lists_unique = true;
  g3m3::InnerOrder inner_order[G3M3_MAX_GRIDS];   // per box: how its inner-boundary lists must be applied
  int* ij[3] = {};
  float* parm[3] = {};
  int num[3][G3M3_MAX_GRIDS] = {};
  int mlen[3] = {};
  bool inner_set = false;
  bool inner_in_shell = true;        // an inner-boundary cell lies in the two-cell flank shell
  float *efld[3], *curr[3], *bs[3], *btot, *ev[3], *tv[3], *vt[3];
  float* glist = nullptr;
  float* flank_ibuf = nullptr;       // interpolated flank values of a box-step [field][shell cell]
  size_t gcap = 0;
  unsigned* words = nullptr;         // [0] list count, [1..5] maxima scratch, [8+5b..] per-box maxima
  unsigned* host_words = nullptr;
  g3m3::CgState* cg = nullptr;
  g3m3::CgState* host_cg = nullptr;
  float* cgvec = nullptr;
  // div B of all boxes at once: per-box solver state, vectors (box 1 uses
  // cgvec) and streams, made at the first pass
  g3m3::CgState* cg_box = nullptr;
  g3m3::CgState* host_cg_box = nullptr;
  float* cgvec_more = nullptr;
  cudaStream_t divb_stream[G3M3_MAX_GRIDS] = {};
  cudaEvent_t divb_ev[G3M3_MAX_GRIDS] = {};
  int cg_hint_box[G3M3_MAX_GRIDS] = {};
  g3m3::CgRun divb_run[G3M3_MAX_GRIDS];      // the pass in flight (divb_begin / divb_poll / divb_end)
  int divb_rep[G3M3_MAX_GRIDS] = {};
  bool divb_fin[G3M3_MAX_GRIDS] = {};
  int divb_worst = 0;
  // host-fed step (g3m3_model_step_host): the state to upload while the
  // next step is enqueued, box by box on a copy stream
  const float* up_src = nullptr;
  bool up_waited[G3M3_MAX_GRIDS] = {};
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t up_fork = nullptr, up_ev[G3M3_MAX_GRIDS] = {};
  float* d_scal = nullptr;
  float* h_scal = nullptr;
  int nscal = 0, scal_cap = 0;
  double t = 0.0;
  double t_old[G3M3_MAX_GRIDS] = {}, t_new[G3M3_MAX_GRIDS] = {};
  double t_step[G3M3_MAX_GRIDS] = {}, t_stepnew[G3M3_MAX_GRIDS] = {};
  int64_t cell_updates = 0;
  int nsteps_done = 0;
  float iso_flag = 1.0f;
  int64_t kernels = 0, graph_launches = 0;
  std::vector<int> h_ij[3];          // host copies of the inner-boundary tables (fluid files)
  std::vector<float> h_parm[3];
  int fcs_variant = 0;               // fcsmooth tile shape (g3m3_model_autotune)
  int contracted = 0;                // the contracted flavour of the hot kernels (g3m3_model_set_contracted)
  float* flux_hist = nullptr;        // flux_counter history [step][box][6]
  unsigned* flux_count = nullptr;
  int flux_cap = 0;
  float flux_scale[G3M3_MAX_GRIDS] = {};
  float* craft_traj = nullptr;       // virtual spacecraft: trajectories (4, samples)
  int* craft_start = nullptr;        // first sample of each craft
  float* craft_out = nullptr;        // records [step][craft][4 + nf]
  unsigned* craft_count = nullptr;
  int ncraft = 0, craft_nf = 0, craft_cap = 0, craft_t_slot = -1;
  int craft_fields[8] = {};
  std::map<std::string, cudaGraphExec_t> graphs;
  std::map<std::string, int> plan_seen;   // host-launched sightings of a step plan not yet captured
  int capture_after = 1;                  // capture a plan's graph at its n-th sighting
  std::map<std::string, int64_t> kernel_nodes;
  int64_t launches_in_step = 0;
  // adjoint recording (adjoint.cu): when set, every box-step, core sync
  // and final sync of a main step leaves the snapshots its reverse needs
  g3m3::Tape* tape = nullptr;
  // a prescribed time-step schedule: t_stepnew of every box at the start
  // of each of the next forced_n main steps (the adjoint holds dt fixed)
  const double* forced_steps = nullptr;
  int forced_n = 0, forced_i = 0;
};

namespace g3m3 {
// Tape hooks, implemented in adjoint.cu; the engine calls them only while
// m->tape is set.  fields: the 34 field pointers of the box's state.
void tape_box_start(g3m3_model* m, int box, float dt2, float dt, float t1p, float t1c);
void tape_snap(g3m3_model* m, int point, int box, float* const fields[G3M3_NFIELDS]);
void tape_core(g3m3_model* m, int box);
void tape_final(g3m3_model* m, int box);   // after the final sync's corer, before its set_rho
void tape_divb(g3m3_model* m);
// engine.cu: the fields stage and fnd_vtot of an explicit table of 34 box
// fields, on the model's stream, into the model's scratch
void engine_fields(g3m3_model* m, float* const f[G3M3_NFIELDS], int b);
void engine_vtot(g3m3_model* m, float* const f[G3M3_NFIELDS]);
}  // namespace g3m3
