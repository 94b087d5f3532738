// Dispatch of the per-position kernels on the region-of-interest shape. The
// fused kernels are templates in ptycho_position.cuh, instantiated once per
// shape in ptycho_position_<S>.cu (square) and ptycho_position_<SX>x<SY>.cu;
// 256 x 256 runs the batch-wide kernels of ptycho_staged.cu.
#include <cuda_runtime.h>

#include "ptycho_internal.h"

namespace pty {

#define PTY_DECLARE_SIZE(S)                                                         \
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
PTY_DECLARE_SIZE(96x128)
PTY_DECLARE_SIZE(128x96)

namespace {
constexpr int roi_key(int sx, int sy) { return sx * 4096 + sy; }
}  // namespace

bool roi_supported(int Sx, int Sy) {
  switch (roi_key(Sx, Sy)) {
    case roi_key(32, 32):
    case roi_key(48, 48):
    case roi_key(64, 64):
    case roi_key(96, 96):
    case roi_key(128, 128):
    case roi_key(96, 128):
    case roi_key(128, 96):
    case roi_key(256, 256):
      return true;
    default:
      return false;
  }
}

#define PTY_DISPATCH(FN, A, S)                                  \
  switch (roi_key((A).Sx, (A).Sy)) {                            \
    case roi_key(32, 32): return FN##_32(A, S);                 \
    case roi_key(48, 48): return FN##_48(A, S);                 \
    case roi_key(64, 64): return FN##_64(A, S);                 \
    case roi_key(96, 96): return FN##_96(A, S);                 \
    case roi_key(128, 128): return FN##_128(A, S);              \
    case roi_key(96, 128): return FN##_96x128(A, S);            \
    case roi_key(128, 96): return FN##_128x96(A, S);            \
    default: return cudaErrorInvalidValue;                      \
  }

// (the staged path has no position correction and no exact probe gradient:
// the C ABI refuses both for 256 x 256 and resampled batches)
// The probe spectrum of every ROI shape: two passes of line transforms over all
// modes, many blocks each (ptycho_staged.cu), which also publish the twiddle
// tables the fused kernels read. Same passes and twiddles as the fused kernels'
// 2D transform, so the spectrum has the same bits as one block's would.
cudaError_t launch_probe_spectrum(const BatchArgs& a, cudaStream_t s) {
  return launch_staged_spectrum(a, s);
}

cudaError_t launch_position_kernel(const BatchArgs& a, cudaStream_t s) {
  if (staged_batch(a)) return launch_staged_positions(a, s);
  PTY_DISPATCH(launch_position_kernel, a, s)
}

cudaError_t launch_position_correction(const BatchArgs& a, cudaStream_t s) {
  if (staged_roi(a.Sx, a.Sy)) return cudaErrorNotSupported;
  PTY_DISPATCH(launch_position_correction, a, s)
}

cudaError_t launch_probe_inverse(const BatchArgs& a, cudaStream_t s) {
  if (staged_roi(a.Sx, a.Sy)) return cudaErrorNotSupported;
  PTY_DISPATCH(launch_probe_inverse, a, s)
}

cudaError_t launch_probe_intensity(const BatchArgs& a, cudaStream_t s) {
  if (staged_roi(a.Sx, a.Sy)) return launch_staged_intensity(a, s);
  PTY_DISPATCH(launch_probe_intensity, a, s)
}

cudaError_t launch_probe_aperture(const BatchArgs& a, cudaStream_t s) {
  if (staged_roi(a.Sx, a.Sy)) return launch_staged_aperture(a, s);
  PTY_DISPATCH(launch_probe_aperture, a, s)
}

}  // namespace pty
