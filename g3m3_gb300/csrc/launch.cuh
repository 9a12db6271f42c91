// launch.cuh -- host-side launch helpers and the kernel launcher
// declarations shared by the C ABI and the step engine.
#pragma once

#include "device.cuh"
#include "kargs.cuh"

namespace g3m3 {

inline dim3 grid3(const Dims& d, const dim3& blk) {
  return dim3((unsigned)((d.nx + blk.x - 1) / blk.x), (unsigned)((d.ny + blk.y - 1) / blk.y),
              (unsigned)((d.nz + blk.z - 1) / blk.z));
}

inline unsigned blocks_for(size_t n, unsigned threads) {
  return (unsigned)((n + threads - 1) / threads);
}

// k_push.cu
void launch_flux_counter(const FluxArgs& a, cudaStream_t s);
void launch_craft(const CraftArgs& a, cudaStream_t s);
void launch_init(const InitArgs& a, cudaStream_t s);
void launch_velocity_floor(const float* rho, const float* const p[3], float* const v[3], float floor_, size_t n,
                           cudaStream_t s);
void launch_cut(const CutArgs& a, cudaStream_t s);
void launch_push_ion(const PushIonArgs& a, cudaStream_t s);
void launch_push_field(const PushFieldArgs& a, cudaStream_t s);
// k_fields.cu
void launch_current(const CurrentArgs& a, cudaStream_t s);
void launch_evel(const EvelArgs& a, cudaStream_t s);
void launch_bande(const BandEArgs& a, cudaStream_t s);
void launch_bande_list(const BandEListArgs& a, cudaStream_t s);
void launch_bande_faces(float* const efld[3], const Dims& d, cudaStream_t s);
void launch_fnd_pres(const float* const pr[3], float* p_para, float* p_perp, float* p_cross,
                     const float* const v[3], const float* const b[3], const Dims& d,
                     cudaStream_t s);
void launch_total_b(const float* const b[3], const float* const b0[3], float* const bs[3],
                    float* btot, float smallbit, const Dims& d, cudaStream_t s);
// k_smooth.cu
void launch_lap(const LapArgs& a, cudaStream_t s);
void launch_vtot(const VtotArgs& a, cudaStream_t s);
void launch_fcsmooth(const FcsArgs& a, cudaStream_t s);
cudaError_t prepare_fcsmooth();   // once, outside stream capture
// k_guards.cu
void launch_guards(const GuardArgs& a, cudaStream_t s);
void launch_guard_scatter(const ScatterArgs& a, cudaStream_t s);
// set_speed_agrd's maxima where one met a NaN, in the reference's loop order
// (GuardArgs::fold): the species words before the scatter, alfmax after it
void launch_guard_fold_species(const GuardArgs& a, cudaStream_t s);
void launch_guard_fold_alf(const GuardArgs& a, cudaStream_t s);
void launch_copy(float* dst, const float* src, size_t n, cudaStream_t s);

}  // namespace g3m3
