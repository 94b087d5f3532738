// Internal declarations shared by the kernel and C-ABI translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace pty {

constexpr int kTile = 16;          // object reduction tile (kTile x kTile pixels)
constexpr int kProbeChunks = 16;   // batch chunks of the probe-gradient reduction
constexpr int kReduceThreads = 256;

// Per-batch kernel arguments (device pointers into caller buffers/workspace).
struct BatchArgs {
  int Sx, Sy, Px, Py, T, M;
  int Ax, Ay;              // detector (amplitude) shape; = Sx, Sy without resampling
  int resample;            // far field resampled between the ROI and the detector grid
  int potential;           // object is float32 potential
  int projection;          // projection-set update instead of gradient descent
  int mixed_formula;       // |F|_tot ratio form (mixed-state class)
  int B;
  float step, norm_min;
  float pa, pb, pc;        // projection parameters a, b, c
  int fix_probe;
  int ew_valid;
  int staging_t;           // staged per-position terms are y-major (e' = y * Sx + x)
  int forward_only;        // forward model and per-position error only, no adjoint
  int keep_farfield;       // single slice: keep FFT2(psi_m) of each position in scratch_f
  int exact_probe_grad;    // probe term through the adjoint of the sub-pixel shift
  int prepare_spectrum;    // after the probe update, the next batch's probe spectrum
  int nobj_only;           // object reduction of the |P|^2 terms alone (probe overlap)
  int nprobe_from_object;  // plain single-slice GD: the probe side gathers |O|^2 from the
                           // object instead of reading staged terms (none are written)
  const float* aperture;   // (N) Fourier amplitude of the initial probe (aperture constraint)

  void* object;                 // (T,Px,Py) float2 or float
  float2* probe;                // (M,N)
  const float* amplitudes;      // (J,N)
  const int32_t* amp_rows;      // (B) or null
  const float* positions;       // (J,2)
  const int32_t* pos_rows;      // (B) or null
  const float* det_mask;        // (N) or null
  const float2* props;          // (T-1,N) or null
  float2* exit_waves;           // (J,M,N) or null
  float* error_accum;           // scalar

  // position correction (after the batch update; positions_rw is the positions
  // array above, updated in place)
  float* positions_rw;             // (J,2)
  const float* positions_initial;  // (J,2)
  float pc_step;                   // positions_step_size
  double pc_max_update;            // pixels; < 0: no limit
  double pc_max_total;             // pixels; < 0: no limit

  // workspace
  float2* probe_spec;   // (M,N)
  float2* tw;           // (Sx + Sy) twiddle tables exp(-2 pi i m / S), x then y
  float2* st_obj;       // (T,B,N)
  float* st_nobj;       // (T,B,N)
  float2* st_probe;     // (B,M,N)
  float* st_nprobe;     // (B,N)
  float2* scratch_f;    // (B,M,N) far fields FFT2(psi_m): single slice, or kept for A16
  float2* st_pm;        // (T,B,M,N) probe of each slice and mode (mixed-state multislice)
  int2* pos_round;      // (B)
  float* err;           // (B)
  float* err_part;      // (B, chunks) per-chunk error partials of the staged path
  float2* det_f;        // (B,M,Ax Ay) detector-grid far fields (resampling only)
  float2* obj_grad;     // (T,P)
  float* obj_nrm;       // (T,P)
  float* tile_max;      // (T,ntiles)
  float2* probe_part;   // (chunks,M,N)
  float* probe_npart;   // (chunks,N)
  float* probe_bmax;    // (N/256)
  float2* probe_grad;   // (M,N)
  float* probe_nrm;     // (N)
  double* com;          // (4) scratch for the probe CoM constraint
  float* red;           // (1024) scratch for constraint reductions
};

struct Workspace {
  size_t probe_spec, tw, st_obj, st_nobj, st_probe, st_nprobe, scratch_f, st_pm, pos_round, err,
      err_part, det_f, obj_grad, obj_nrm, tile_max, probe_part, probe_npart, probe_bmax,
      probe_grad, probe_nrm, com, red, total;
};

// Ax, Ay: detector shape (resampling when it differs from Sx, Sy)
Workspace workspace_layout(int Sx, int Sy, int Px, int Py, int T, int M, int B,
                           bool keep_farfield, int Ax, int Ay);
void bind_workspace(BatchArgs& a, void* base, const Workspace& w);

bool roi_supported(int Sx, int Sy);

// A scan coordinate as the kernels use it. NaN and infinite coordinates have no
// patch: they are replaced by 0, so every object index derived from them stays
// inside the object, and the kernel reading them marks the position's error NaN
// (reported by ptycho_read_error as PTYCHO_ERR_NONFINITE).
__device__ __forceinline__ float finite_or_zero(float v) { return isfinite(v) ? v : 0.0f; }

// Raises the dynamic shared-memory limit of kernel `fn` to at least `bytes` on
// the current device. Function attributes are per device, so the setting is
// made once per (device, kernel) pair and remembered under a mutex.
cudaError_t ensure_smem_limit(const void* fn, int bytes);

// Position-kernel timing (instrumentation); implemented in ptycho_capi.cu.
void timing_before(cudaStream_t s);
void timing_after(cudaStream_t s);

// Launchers (return cudaError_t of the last launch).
cudaError_t launch_probe_spectrum(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_position_kernel(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_position_correction(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_probe_inverse(const BatchArgs& a, cudaStream_t s);
// |P_b|^2 of the shifted probe (mode 0) of every batch position into st_nobj.
cudaError_t launch_probe_intensity(const BatchArgs& a, cudaStream_t s);
// Probe mode 0 with its Fourier amplitude replaced by a.aperture, power kept.
cudaError_t launch_probe_aperture(const BatchArgs& a, cudaStream_t s);
// Every probe mode times a real-space mask, power of each mode kept.
cudaError_t launch_probe_amplitude(const BatchArgs& a, const float* mask, cudaStream_t s);
// Every slice of the object set to the mean over slices.
cudaError_t launch_identical_slices(const BatchArgs& a, cudaStream_t s);
// Gaussian blur of the object (weights w[0 .. 2R], reflect boundaries), scratch of
// 4 T Px Py floats.
cudaError_t launch_object_gaussian(const BatchArgs& a, const double* w, int R, int pure_phase,
                                   float* scratch, cudaStream_t s);
// overlap += sum over the batch of the staged |P_b|^2, scattered into the object grid.
cudaError_t launch_overlap_accumulate(const BatchArgs& a, float* overlap, cudaStream_t s);
// Register-resident 128 x 128 single-slice GD kernel (ptycho_gd128.cu).
// set_schedule stores the preferred schedule for a ROI edge (0 default,
// 1 shared-memory passes, 2 register-resident, 3 shared-memory passes by groups
// of warps) and returns the previous one; get_schedule reads it.
int set_schedule(int roi, int schedule);
int get_schedule(int roi);
bool position_v2_eligible(const BatchArgs& a);
cudaError_t launch_position_v2(const BatchArgs& a, cudaStream_t s);
// Creates the helper stream and events that batches issued on s use (idempotent).
cudaError_t prepare_stream(cudaStream_t s);
cudaError_t launch_reduce_and_update(const BatchArgs& a, cudaStream_t s);
// Loss and object / probe gradients of a batch (no update); probe_grad may be null.
cudaError_t launch_gradient(const BatchArgs& a, void* object_grad, float2* probe_grad,
                            float* loss, cudaStream_t s);
cudaError_t launch_object_constraints(const BatchArgs& a, const uint8_t* mask,
                                      float shrinkage, int apply_shrinkage,
                                      int pure_phase, int positivity, cudaStream_t s);
cudaError_t launch_probe_com(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_probe_gram(const BatchArgs& a, const float2* probe, float2* gram,
                              cudaStream_t s);
cudaError_t launch_fma_probe(int blocks, int iters, float* sink, cudaStream_t s);
// Gram matrix, device eigen-decomposition and mixing of the probe modes, all on
// stream s (no host round trip; capturable in a CUDA graph).
cudaError_t launch_probe_orthogonalize(const BatchArgs& a, float2* scratch_probe, float2* gram,
                                       float2* coeffs, cudaStream_t s);
cudaError_t launch_probe_mix(const BatchArgs& a, const float2* in, const float2* coeffs,
                             float2* out, cudaStream_t s);

// ---- ptycho_staged.cu: the model as batch-wide kernels (256 x 256 ROI, resampling)
bool staged_roi(int Sx, int Sy);
// the batch runs on the staged path (256 x 256 ROI or a resampled far field)
bool staged_batch(const BatchArgs& a);
// gradient descent or forward only, no kept far fields, no exact probe gradient
bool staged_batch_supported(const BatchArgs& a);
cudaError_t launch_staged_spectrum(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_staged_positions(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_staged_intensity(const BatchArgs& a, cudaStream_t s);
// every probe mode shifted by -a.com (after probe_com_kernel)
cudaError_t launch_staged_probe_shift(const BatchArgs& a, cudaStream_t s);
cudaError_t launch_staged_aperture(const BatchArgs& a, cudaStream_t s);

// Preprocessing kernels (ptycho_preprocess.cu).
cudaError_t launch_pattern_com(const float* in, int num, int Qx, int Qy, const void* mask,
                               int mask_mode, void* cx, void* cy, cudaStream_t s);
cudaError_t launch_rotation_search(const void* nx, const void* ny, int R0, int R1,
                                   const float* cos_a, const float* sin_a, int A, int div,
                                   int is_double, void* vals, cudaStream_t s);
cudaError_t launch_pattern_normalize(const float* in, int Qx, int Qy, const int32_t* rows,
                                     int num_out, const float* cfx, const float* cfy,
                                     int crop_w, float* amps, float* sums, cudaStream_t s);
// out[i] = src[rows[i]] (pattern_size floats each), at the greatest stream priority
cudaError_t launch_gather_patterns(const float* src, const int32_t* rows, int n, int num_patterns,
                                   int pattern_size, float* dst, cudaStream_t s);

// ---- ptycho_volume.cu (tomography)
cudaError_t launch_volume_rotate(const void* in, int in_is_double, void* out, int out_mode,
                                 int n0, int n1, int n2, const double* matrix,
                                 const double* offset, double* scratch, cudaStream_t s);
cudaError_t launch_volume_project(const float* vol, int n0, size_t P, int T, float* sliced,
                                  cudaStream_t s);
cudaError_t launch_volume_expand(const float* sliced, const float* old, int T, int n0, size_t P,
                                 void* out, int out_mode, cudaStream_t s);
cudaError_t launch_volume_add_scaled(float* vol, const float* addend, size_t n, int divisor,
                                     cudaStream_t s);
cudaError_t launch_volume_constraints(float* vol, size_t n, float shrinkage, int apply_shrinkage,
                                      int positivity, cudaStream_t s);

}  // namespace pty
