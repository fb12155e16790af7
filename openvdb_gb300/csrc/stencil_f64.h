// Host launchers of the FP64 instance (stencil_f64.cu): the RK stage and
// renormalisation kernels on double value buffers (512 doubles per slot),
// buffer conversions, the time step's max |v|^2 in double, and the
// canonical-order gather of the double values.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace gbls {
struct RkArgs;
struct NormArgs;
struct FieldParams;

void launch_rk_f64(const RkArgs& a, cudaStream_t s);
void launch_norm_f64(const NormArgs& a, cudaStream_t s);
// out[i] = double(in[i]) / float(in[i]) (round to nearest) for i < n
void launch_widen(const float* in, double* out, size_t n, cudaStream_t s);
void launch_narrow(const double* in, float* out, size_t n, cudaStream_t s);
// |v|^2 in double of the first active voxel (leaf order, voxel order) whose
// Vec3f |v|^2 equals maxv2, into *out (-1 when none); argkey is scratch.
void launch_argmax_f64(int64_t nleaf, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                       const FieldParams& f, float t0, float maxv2, unsigned long long* argkey, double* out,
                       cudaStream_t s);
// out[prefix[l] + rank] = vals[slot[l] * 512 + rank] over the active voxels
void launch_gather_active_f64(int64_t n, const int32_t* slot, const uint64_t* am, const int64_t* prefix,
                              const double* vals, double* out, cudaStream_t s);
}  // namespace gbls
