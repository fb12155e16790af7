// Host launchers of the stencil kernels (one set per arithmetic policy).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace gbls {
struct RkArgs;
struct NormArgs;
struct CflArgs;

// Bit-faithful to the reference arithmetic (FP64 WENO weights).
void launch_rk_parity(const RkArgs& a, cudaStream_t s);
void launch_norm_parity(const NormArgs& a, cudaStream_t s);
// The same bits as the parity launchers on the FP32 pipes (ExactArith).
void launch_rk_exact(const RkArgs& a, cudaStream_t s, int min_ctas = 0);
void launch_norm_exact(const NormArgs& a, cudaStream_t s, int min_ctas = 0);
// ExactArith's WENO5 on n quintuples (device arrays; decided may be null).
void launch_weno5_exact(const float* v, int64_t n, float* out, uint8_t* decided, cudaStream_t s);
// FP32 arithmetic.
void launch_rk_fast(const RkArgs& a, cudaStream_t s);
void launch_norm_fast(const NormArgs& a, cudaStream_t s);
// Max |v|^2 over active voxels (exact in both modes).
// leaves_per_block: 8, 16, 32 (default) or 64 leaves per CTA, 8 threads each
void launch_cfl(const CflArgs& a, cudaStream_t s, int leaves_per_block = 32);
// LevelSetMorphing: speed sampling (+ max |s| into *max_bits) and RK stages.
struct MorphSpeedArgs;
struct MorphArgs;
void launch_morph_speed_parity(const MorphSpeedArgs& a, unsigned int* max_bits, cudaStream_t s);
void launch_morph_stage_parity(const MorphArgs& a, cudaStream_t s);
void launch_morph_speed_fast(const MorphSpeedArgs& a, unsigned int* max_bits, cudaStream_t s);
void launch_morph_stage_fast(const MorphArgs& a, cudaStream_t s);
void launch_morph_stage_exact(const MorphArgs& a, cudaStream_t s);
// LevelSetFilter passes.
struct FilterArgs;
void launch_filter_parity(const FilterArgs& a, cudaStream_t s);
void launch_filter_fast(const FilterArgs& a, cudaStream_t s);
void launch_filter_exact(const FilterArgs& a, cudaStream_t s);
}  // namespace gbls
