// Dispatch of the fused per-position kernels on the region-of-interest edge.
// The kernels are templates in ptycho_position.cuh, instantiated once per edge
// in ptycho_position_<S>.cu.
#include <cuda_runtime.h>

#include "ptycho_internal.h"

namespace pty {

#define PTY_DECLARE_SIZE(S)                                                         \
  cudaError_t launch_probe_spectrum_##S(const BatchArgs& a, cudaStream_t s);        \
  cudaError_t launch_position_kernel_##S(const BatchArgs& a, cudaStream_t s);       \
  cudaError_t launch_position_correction_##S(const BatchArgs& a, cudaStream_t s);   \
  cudaError_t launch_probe_inverse_##S(const BatchArgs& a, cudaStream_t s);         \
  cudaError_t launch_probe_intensity_##S(const BatchArgs& a, cudaStream_t s);        \
  cudaError_t launch_probe_aperture_##S(const BatchArgs& a, cudaStream_t s);

PTY_DECLARE_SIZE(32)
PTY_DECLARE_SIZE(48)
PTY_DECLARE_SIZE(64)
PTY_DECLARE_SIZE(96)
PTY_DECLARE_SIZE(128)

bool roi_supported(int Sx, int Sy) {
  if (Sx != Sy) return false;
  switch (Sx) {
    case 32:
    case 48:
    case 64:
    case 96:
    case 128:
      return true;
    default:
      return false;
  }
}

#define PTY_DISPATCH(FN, A, S)                 \
  switch ((A).Sx) {                            \
    case 32: return FN##_32(A, S);             \
    case 48: return FN##_48(A, S);             \
    case 64: return FN##_64(A, S);             \
    case 96: return FN##_96(A, S);             \
    case 128: return FN##_128(A, S);           \
    default: return cudaErrorInvalidValue;     \
  }

cudaError_t launch_probe_spectrum(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_probe_spectrum, a, s)
}

cudaError_t launch_position_kernel(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_position_kernel, a, s)
}

cudaError_t launch_position_correction(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_position_correction, a, s)
}

cudaError_t launch_probe_inverse(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_probe_inverse, a, s)
}

cudaError_t launch_probe_intensity(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_probe_intensity, a, s)
}

cudaError_t launch_probe_aperture(const BatchArgs& a, cudaStream_t s) {
  PTY_DISPATCH(launch_probe_aperture, a, s)
}

}  // namespace pty
