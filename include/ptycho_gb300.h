/*
 * ptycho_gb300.h — C ABI of the GB300 (sm_103a) iterative-ptychography kernels.
 *
 * One shared library (libptycho_gb300.so) exports these entry points. They
 * replace the array operations the py4DSTEM 0.14.18 reconstruction classes run
 * per position batch and per iteration on their CuPy path (the reference has no
 * native code for this path: every operator is NumPy/CuPy array code, so each
 * entry point cites the reference Python function whose work it performs).
 *
 * Conventions
 *  - All array arguments are DEVICE pointers, row-major, densely packed.
 *    Complex arrays are interleaved complex64 (float re, float im).
 *  - Shapes: probe/detector ROI (Sx, Sy); object (T, Px, Py); probe (M, Sx, Sy);
 *    amplitudes (J, Sx, Sy) float32, corner-centred; positions (J, 2) float32
 *    in object pixels.
 *  - "rows" arrays (int32, length batch) select, for batch position b, the
 *    pattern / position / exit wave row used; NULL means row b.
 *  - Every call is asynchronous on `stream` (a cudaStream_t, NULL = legacy
 *    default stream) and allocates nothing: scratch space is the caller's
 *    `workspace` of at least ptycho_workspace_bytes() bytes, 256-byte aligned.
 *  - Return value: PTYCHO_OK (0) or an error code; ptycho_last_error() gives a
 *    message (per host thread). No C++ exception crosses this boundary.
 *  - Results are deterministic for a given geometry and batch size: gradient
 *    sums over positions use fixed-order, position-tiled reductions, no float
 *    atomics.
 */
#ifndef PTYCHO_GB300_H
#define PTYCHO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTYCHO_ABI_VERSION 5

enum ptycho_status {
  PTYCHO_OK = 0,
  PTYCHO_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size or flag          */
  PTYCHO_ERR_UNSUPPORTED = 2,      /* ROI size or geometry without a kernel   */
  PTYCHO_ERR_WORKSPACE = 3,        /* workspace too small or misaligned       */
  PTYCHO_ERR_CUDA = 4,             /* a CUDA launch or runtime call failed    */
  PTYCHO_ERR_NONFINITE = 5         /* a reduction produced NaN or Inf         */
};

/* Geometry shared by every call of one reconstruction. */
typedef struct ptycho_geometry {
  int32_t roi_x;               /* Sx: probe / detector pixels along x         */
  int32_t roi_y;               /* Sy                                          */
  int32_t object_x;            /* Px (>= Sx)                                  */
  int32_t object_y;            /* Py (>= Sy)                                  */
  int32_t num_slices;          /* T: 1 = single slice                         */
  int32_t num_probes;          /* M: 1 = single probe                         */
  int32_t object_is_potential; /* 0: complex64 object, 1: float32 potential   */
  int32_t flags;               /* PTYCHO_FLAG_* bits; unknown bits must be 0  */
  int32_t detector_x;          /* Ax: detector pixels along x; 0 = roi_x       */
  int32_t detector_y;          /* Ay; 0 = roi_y                                */
} ptycho_geometry;

/* A detector shape (Ax, Ay) different from the ROI (Sx, Sy) is the reference's
 * region_of_interest_shape (singleslice_ptychography.py:431-436): the
 * amplitudes and the detector mask are Ax x Ay, and every Fourier projection
 * resamples the far field onto the detector grid and the modified far field
 * back onto the ROI grid as the reference's bilinear_resample does
 * (ptychographic_methods.py:1601-1631, utils.py:2347-2428; SciPy's zoom of a
 * complex array maps output index k to input coordinate
 * k (n_in - 1) / (n_out - 1), linear between neighbours, and the sums are
 * kept by dividing by the ratio of pixel counts). Gradient descent of every
 * model, the self-consistency errors and the object gradient; projection sets,
 * PTYCHO_FLAG_KEEP_FARFIELD (position correction) and the probe gradient are
 * refused with PTYCHO_ERR_UNSUPPORTED. */

/* Use the mixed-state Fourier projection (shared ratio A/sqrt(sum_m |F_m|^2),
 * mixedstate class) even when num_probes == 1. Implied when num_probes > 1. */
#define PTYCHO_FLAG_MIXED_STATE 1

/* Keep each position's far field FFT2(psi) of the forward pass (psi the exit
 * wave of every probe mode) in the workspace for a following
 * ptycho_position_correction() call. Gradient descent and projection sets, any
 * model (projection sets transform psi once more per position and mode). */
#define PTYCHO_FLAG_KEEP_FARFIELD 2

/* Batch chaining within one iteration (batch calls on one workspace and stream):
 * PTYCHO_FLAG_PREPARE_SPECTRUM: after the probe update, compute the spectrum of
 * the updated probe into the workspace (on the helper stream, concurrently with
 * the object update) for the next batch call;
 * PTYCHO_FLAG_SPECTRUM_READY: the workspace already holds the spectrum of the
 * current probe (prepared by the previous batch call, or the probe is fixed),
 * so the call skips its own. The probe must not change in between. */
#define PTYCHO_FLAG_SPECTRUM_READY 4
#define PTYCHO_FLAG_PREPARE_SPECTRUM 8

/* Library identity and capability queries. */
int ptycho_abi_version(void);
const char* ptycho_last_error(void);
/* 1 if kernels exist for this ROI (Sx, Sy), else 0: the fused per-position
 * kernel for square 32, 48, 64, 96, 128 and 96 x 128, 128 x 96 (every model);
 * batch-wide staged kernels for 256 x 256 (gradient descent of every model,
 * the self-consistency errors and the object gradient; projection sets,
 * PTYCHO_FLAG_KEEP_FARFIELD and the probe gradient are refused). */
int ptycho_roi_supported(int32_t roi_x, int32_t roi_y);
/* PTYCHO_OK if the batch entry points take this geometry, else the error code
 * (PTYCHO_ERR_UNSUPPORTED or PTYCHO_ERR_INVALID_ARGUMENT) they would return,
 * with the reason in ptycho_last_error(). Host only; touches no device. */
int ptycho_geometry_supported(const ptycho_geometry* geometry);

/* Scratch bytes one batch call needs for up to max_batch positions. */
size_t ptycho_workspace_bytes(const ptycho_geometry* geometry, int32_t max_batch);

/*
 * One gradient-descent batch: forward model, Fourier amplitude projection,
 * adjoint and the object/probe update, for `batch` positions.
 *
 * Replaces, per batch of reconstruct() (singleslice_ptychography.py:859-929,
 * multislice_ptychography.py:975-1047, mixedstate_ptychography.py:889-957):
 *   fft_shift / _return_shifted_probes  (utils.py:508-533, ptychographic_methods.py:1482-1487)
 *   _overlap_projection                 (ptychographic_methods.py:1489-1527, 2300-2351, 2696-2734)
 *   _gradient_descent_fourier_projection (ptychographic_methods.py:1576-1635, 2742-2804)
 *   _gradient_descent_adjoint           (ptychographic_methods.py:1818-1908, 2353-2458, 2906-3000)
 *   _sum_overlapping_patches_bincounts  (phase_base_class.py:1905-1968)
 * object: (T,Px,Py) complex64, or float32 if object_is_potential.
 * probe: (M,Sx,Sy) complex64, updated unless fix_probe.
 * detector_mask: (Sx,Sy) float32 corner-centred Fourier mask or NULL.
 * propagators: (T-1,Sx,Sy) complex64 Fresnel propagators (NULL when T == 1).
 * error_accum: one float32 on the device; the batch error sum is added to it.
 */
int ptycho_gd_batch(const ptycho_geometry* geometry, void* object, void* probe,
                    const float* amplitudes, const int32_t* amplitude_rows,
                    const float* positions_px, const int32_t* position_rows,
                    int32_t batch, float step_size, float normalization_min,
                    int32_t fix_probe, const float* detector_mask,
                    const void* propagators, float* error_accum, void* workspace,
                    size_t workspace_bytes, void* stream);

/*
 * One projection-set batch (DM_AP, RAAR, RRR, SUPERFLIP, generalized (a,b,c)):
 * exit-wave update and the ASSIGNED (not accumulated) object/probe estimates.
 * Replaces _projection_sets_fourier_projection (ptychographic_methods.py:1637-1734,
 * 2806-2904) and _projection_sets_adjoint (1910-1998, 2460-2565, 3002-3093).
 * exit_waves: (J,M,Sx,Sy) complex64 persistent state indexed by position_rows;
 * exit_waves_valid = 0 on the first iteration (the overlap seeds them).
 */
int ptycho_projection_batch(const ptycho_geometry* geometry, void* object, void* probe,
                            const float* amplitudes, const int32_t* amplitude_rows,
                            const float* positions_px, const int32_t* position_rows,
                            int32_t batch, float projection_a, float projection_b,
                            float projection_c, float normalization_min,
                            int32_t fix_probe, void* exit_waves,
                            int32_t exit_waves_valid, const void* propagators,
                            float* error_accum, void* workspace,
                            size_t workspace_bytes, void* stream);

/*
 * Position correction of the batch just updated by ptycho_gd_batch() (called
 * with PTYCHO_FLAG_KEEP_FARFIELD, the same geometry, workspace, amplitudes,
 * rows and batch, and no other batch call on that workspace in between).
 * Replaces _position_correction (ptychographic_methods.py:2071-2225): per
 * position a 2x2 least-squares shift from the intensity change of one-pixel
 * object shifts, using the object after the update, scaled by step_size,
 * limited to max_update_px per call and to max_total_px from positions_initial
 * (negative = no limit; pixels), and subtracted from positions_px[row] in place.
 * The perturbed waves start, as in the reference, from the batch's shifted
 * probes (single slice, mixed state) or from the updated unshifted probe
 * propagated through all slices (multislice, multislice_ptychography.py:1026-1038;
 * probe and propagators are read only then). A position whose 2x2 system is
 * singular keeps its place (the reference raises LinAlgError).
 */
int ptycho_position_correction(const ptycho_geometry* geometry, const void* object,
                               const void* probe, const void* propagators,
                               const float* amplitudes, const int32_t* amplitude_rows,
                               float* positions_px, const float* positions_initial,
                               const int32_t* position_rows, int32_t batch, float step_size,
                               double max_update_px, double max_total_px, void* workspace,
                               size_t workspace_bytes, void* stream);

/*
 * Loss and gradients of one batch, without an update (the backward of an
 * autograd function over the forward model). loss[0] = sum over the batch of
 * sum_k (A - |F|)^2 (the batch error of _gradient_descent_fourier_projection,
 * ptychographic_methods.py:1576-1635, 2742-2804); object_grad (T,Px,Py) complex64
 * (float32 for potentials) and probe_grad (M,Sx,Sy) complex64 (NULL: skipped)
 * receive dloss/dRe + i dloss/dIm (for potentials dloss/dV). The object gradient
 * is -2N times the summed adjoint terms of _gradient_descent_adjoint
 * (ptychographic_methods.py:1818-1908, 2353-2458, 2906-3000, 3162-3400) before their
 * normalisation and step. The probe gradient is exact: each position's term
 * conj(O) chi goes back through the adjoint of its sub-pixel shift before the sum
 * (the reference's probe update sums the unshifted terms).
 */
int ptycho_gd_gradient(const ptycho_geometry* geometry, const void* object, const void* probe,
                       const float* amplitudes, const int32_t* amplitude_rows,
                       const float* positions_px, const int32_t* position_rows, int32_t batch,
                       const float* detector_mask, const void* propagators, void* object_grad,
                       void* probe_grad, float* loss, void* workspace, size_t workspace_bytes,
                       void* stream);

/*
 * Per-position self-consistency error sum_k (A - |F|)^2 of a forward-only pass
 * (no update), written to errors[b] for the `batch` positions. Replaces the
 * per-batch body of _return_self_consistency_errors
 * (ptychographic_methods.py:2227-2291); the caller divides by the mean
 * intensity. No detector mask (the reference applies none here).
 */
int ptycho_self_consistency_errors(const ptycho_geometry* geometry, const void* object,
                                   const void* probe, const float* amplitudes,
                                   const int32_t* amplitude_rows, const float* positions_px,
                                   const int32_t* position_rows, int32_t batch,
                                   const void* propagators, float* errors, void* workspace,
                                   size_t workspace_bytes, void* stream);

/*
 * Per-iteration object constraints, default-on subset: shrinkage by
 * shrinkage_rad plus the mean phase (or potential) over `mask` (Px,Py uint8,
 * NULL = no mask term), then amplitude threshold |O| <= 1 (pure_phase: |O| = 1)
 * for complex objects or positivity for potentials.
 * Replaces _object_shrinkage_constraint / _object_threshold_constraint /
 * _object_positivity_constraint (ptychographic_constraints.py:29-117, 411-464).
 */
int ptycho_object_constraints(const ptycho_geometry* geometry, void* object,
                              const uint8_t* mask, float shrinkage_rad,
                              int32_t apply_shrinkage, int32_t pure_phase,
                              int32_t positivity, void* workspace,
                              size_t workspace_bytes, void* stream);

/*
 * Probe centre-of-mass constraint: Fourier-shift every mode so that the
 * intensity centre of mass of mode 0 sits at the corner origin.
 * Replaces _probe_center_of_mass_constraint (ptychographic_constraints.py:894-918,
 * 1156-1179).
 */
int ptycho_probe_com_constraint(const ptycho_geometry* geometry, void* probe,
                                void* workspace, size_t workspace_bytes, void* stream);

/*
 * Mixed-state orthogonalisation, step 1: the M x M Gram matrix
 * gram[i*M+j] = sum conj(P_i) P_j (complex64, full matrix).
 * Replaces the pairwise products of _probe_orthogonalization_constraint
 * (ptychographic_constraints.py:1181-1216).
 */
int ptycho_probe_gram(const ptycho_geometry* geometry, const void* probe, void* gram,
                      void* stream);

/*
 * Mixed-state orthogonalisation, step 2: probe_out[i] = sum_j coeffs[i*M+j] * probe_in[j]
 * (complex64 coefficients; the eigenvector transform and the intensity sort are
 * folded into `coeffs` by the caller). probe_out must not alias probe_in.
 */
int ptycho_probe_mix(const ptycho_geometry* geometry, const void* probe_in,
                     const void* coeffs, void* probe_out, void* stream);

/*
 * Mixed-state orthogonalisation entirely on the device (for graph capture):
 * Gram matrix, eigen-decomposition of the M x M Hermitian matrix (cyclic Jacobi
 * in double, M <= 16) and mixing, in place on `probe`. Modes come out ordered by
 * decreasing intensity like _probe_orthogonalization_constraint
 * (ptychographic_constraints.py:1181-1216); each eigenvector's phase is fixed so
 * that its largest component is real and positive, so the modes may differ from
 * the reference's LAPACK eigenvectors by a constant phase per mode (to which the
 * mixed-state model is invariant).
 */
int ptycho_probe_orthogonalize(const ptycho_geometry* geometry, void* probe, void* workspace,
                               size_t workspace_bytes, void* stream);

/*
 * Optional per-iteration constraints (off by default in the reference).
 *
 * Identical slices: every slice of the (T, Px, Py) object becomes the mean over
 * slices. Replaces _object_identical_slices_constraint
 * (ptychographic_constraints.py:630-647).
 */
int ptycho_object_identical_slices(const ptycho_geometry* geometry, void* object, void* stream);

/*
 * Gaussian object constraint: the object (all axes of the (T, Px, Py) array, the
 * real and imaginary parts separately; the phase alone with pure_phase) blurred
 * with weights[0 .. 2 radius] (float64, the normalised Gaussian) and reflecting
 * boundaries, one axis after the other, each pass in float64 and stored as
 * float32. scratch: 4 T Px Py floats. Replaces _object_gaussian_constraint
 * (ptychographic_constraints.py:119-151, scipy.ndimage.gaussian_filter).
 */
int ptycho_object_gaussian_constraint(const ptycho_geometry* geometry, void* object,
                                      const double* weights, int32_t radius,
                                      int32_t pure_phase, void* scratch, void* stream);

/*
 * Probe aperture: probe mode 0 <- IFFT2(exp(i angle(FFT2(probe))) aperture), scaled
 * back to its power sum |probe|^2; aperture (Sx, Sy) float32 is the Fourier
 * amplitude of the initial probe. Replaces _probe_aperture_constraint
 * (ptychographic_constraints.py:1004-1040; mode 0 for mixed states, :1243-1247).
 */
int ptycho_probe_aperture_constraint(const ptycho_geometry* geometry, void* probe,
                                     const float* aperture, void* stream);

/*
 * Probe amplitude: every probe mode times the real-space mask (Sx, Sy) float32,
 * scaled back to its power sum. Replaces _probe_amplitude_constraint
 * (ptychographic_constraints.py:920-957); the soft top-hat mask
 * 0.5 (1 - erf(sigma r / (1 - r^2))) is formed by the caller.
 */
int ptycho_probe_amplitude_constraint(const ptycho_geometry* geometry, void* probe,
                                      const float* mask, void* stream);

/*
 * Preprocessing (one-time, before the reconstruction loop). Sums follow the
 * order of NumPy's float32 pairwise add.reduce over each contiguous run, and
 * products and quotients are rounded once each, so the results carry the bits
 * of the reference's float32 NumPy evaluation of the same inputs.
 */

/*
 * Intensity centre of mass of each (qx, qy) pattern of `intensities`
 * (num_patterns, qx, qy) float32: com_x = sum(I kx)/sum(I), com_y = sum(I ky)/sum(I)
 * with kx, ky the pixel indices and I = pattern * mask, in NumPy's types for
 * that product (mask (qx, qy)):
 *   mask_mode 0  no mask (mask NULL); float32 results;
 *   mask_mode 1  float32 mask (a boolean mask as 0/1); float32 results;
 *   mask_mode 2  float64 mask, vectorised form: float64 products, sums and
 *                results (com_x, com_y are double arrays);
 *   mask_mode 3  float64 mask, per-pattern form (the product rounded to float32
 *                in place); float32 results.
 * Replaces the centre of mass of _calculate_intensities_center_of_mass
 * (phase_base_class.py:613-700). Patterns up to 128 x 128 (any shape whose
 * summation tree fits one block's shared memory otherwise).
 */
int ptycho_pattern_com(const float* intensities, int32_t num_patterns, int32_t qx, int32_t qy,
                       const void* mask, int32_t mask_mode, void* com_x, void* com_y,
                       void* stream);

/*
 * Rotation search of the real/reciprocal-space rotation: for every angle a
 * (cos_angles[a], sin_angles[a], float32) and t = 0 (as is) / 1 (x and y
 * exchanged), values[t * num_angles + a] = the mean over the scan interior of
 * |curl| (or |div| when maximize_divergence) of the centre-of-mass field
 * (com_x, com_y) (scan_x, scan_y) rotated by that angle, in float32, or in
 * float64 when com_is_double (com_x, com_y and values are then double arrays,
 * the angles' float32 cos / sin promoted). The caller takes the arg-min
 * (arg-max) exactly as _solve_for_center_of_mass_relative_rotation
 * (phase_base_class.py:1086-1182) does.
 */
int ptycho_rotation_search(const void* com_x, const void* com_y, int32_t com_is_double,
                           int32_t scan_x, int32_t scan_y, const float* cos_angles,
                           const float* sin_angles, int32_t num_angles,
                           int32_t maximize_divergence, void* values, void* stream);

/*
 * Corner-centring and square root: output pattern o takes source pattern
 * rows[o] (rows NULL: pattern o), shifts it periodically and bilinearly by
 * (-com_fitted_x[rows[o]], -com_fitted_y[rows[o]]), writes the sum of the
 * shifted pattern to pattern_sums[o] and sqrt(max(shifted, 0)) to amplitudes
 * (num_out, qx, qy), or, with crop_w > 0, its four crop_w x crop_w corners as a
 * (2 crop_w, 2 crop_w) pattern. The mean diffraction intensity is the float32
 * running sum of pattern_sums in order, divided by num_out. Replaces
 * _normalize_diffraction_intensities (phase_base_class.py:1347-1460).
 * Patterns that fit one block's shared memory are staged there; larger ones
 * (256 x 256) are read from global memory where each value is formed.
 */
int ptycho_normalize_patterns(const float* intensities, int32_t qx, int32_t qy,
                              const int32_t* rows, int32_t num_out, const float* com_fitted_x,
                              const float* com_fitted_y, int32_t crop_w, float* amplitudes,
                              float* pattern_sums, void* stream);

/*
 * Probe-overlap map: overlap (Px, Py) float32 = sum over all positions of
 * |P shifted to the position|^2 scattered into the object grid (probe mode 0,
 * positions in batches of at most max_batch, near-equal sizes, the larger
 * first). The map the preprocessing blurs and thresholds into the object
 * field-of-view mask (singleslice_ptychography.py:504-540). Uses the workspace
 * of ptycho_workspace_bytes(geometry, max_batch).
 */
int ptycho_probe_overlap(const ptycho_geometry* geometry, const void* probe,
                         const float* positions_px, int32_t num_positions, int32_t max_batch,
                         float* overlap, void* workspace, size_t workspace_bytes, void* stream);

/*
 * *device = the device address of host memory [host, host + bytes) when that
 * range is page-locked and mapped (the GPU then reads it in place, over the
 * CPU-GPU link), else NULL. Lets a caller pass host-resident amplitudes to the
 * batch calls without a copy; the reference's storage="cpu" mode keeps them on
 * the host and copies each batch (copy_to_device in reconstruct,
 * singleslice_ptychography.py:873-875).
 */
int ptycho_mapped_host_pointer(const void* host, size_t bytes, void** device);

/*
 * out[i, :] = patterns[rows[i], :] for i < num_out (rows NULL: row i), each
 * pattern pattern_size float32 values; rows is a device array. The per-batch
 * copy of host-resident amplitudes to the device (copy_to_device(
 * self._amplitudes[batch_indices]) in reconstruct,
 * singleslice_ptychography.py:873-875) as one device gather: `patterns` is
 * device memory or the device address of page-locked host memory
 * (ptycho_mapped_host_pointer), read over the CPU-GPU link. The kernel runs at
 * the device's greatest stream priority, so that a gather issued on a second
 * stream for the next batch overlaps the running batch. A row index outside
 * [0, num_patterns) yields a pattern of NaN (the batch error is then
 * non-finite), never an access outside `patterns`.
 */
int ptycho_gather_patterns(const float* patterns, int32_t num_patterns, int64_t pattern_size,
                           const int32_t* rows, int32_t num_out, float* out, void* stream);

/*
 * Creates, for batches issued on `stream`, the helper stream and events on which
 * the probe-side reductions of a batch run concurrently with the object side.
 * A batch call makes them on first use; call this for every stream before
 * capturing batch calls on it in a CUDA graph (creation cannot be captured).
 */
int ptycho_prepare_stream(void* stream);

/*
 * Tomography (PtychographicTomography, ptychographic_tomography.py:991-1240).
 * The object is a (n0, n1, n2) float32 potential volume (z, x, y).
 *
 * ptycho_volume_rotate: out = the volume resampled by the affine map
 * input coordinate = offset + matrix . output coordinate, with cubic B-spline
 * interpolation of mirror-extended spline coefficients and 0 where the input
 * coordinate leaves [0, n - 1] on any axis: scipy.ndimage.affine_transform(order=3,
 * mode="constant", prefilter=True) as _rotate_zxy_volume calls it
 * (ptychographic_methods.py:849-868). Float64 arithmetic throughout. volume is
 * float32 (volume_is_double 0) or float64 (1); out_mode 0 writes float32, 1
 * writes float64, 2 adds into a float32 out (sum in float64, rounded once: the
 * collective update of ptychographic_tomography.py:1121-1124). matrix (9, row
 * major) and offset (3) are host arrays. scratch: n0*n1*n2 doubles. out may be
 * the volume itself.
 */
int ptycho_volume_rotate(const void* volume, int32_t volume_is_double, void* out,
                         int32_t out_mode, int32_t n0, int32_t n1, int32_t n2,
                         const double* matrix, const double* offset, void* scratch,
                         size_t scratch_bytes, void* stream);

/*
 * sliced (num_slices, n1, n2) = the volume summed over consecutive groups of
 * ceil(n0 / num_slices) voxels along z, in voxel order, the last group padded
 * with zeros (_project_sliced_object, ptychographic_methods.py:783-812).
 */
int ptycho_volume_project(const float* volume, int32_t n0, int32_t n1, int32_t n2,
                          int32_t num_slices, float* sliced, void* stream);

/*
 * The voxels of slice t receive (sliced - sliced_old)[t] divided by the number
 * of voxels the slice covers, in float64 (_expand_sliced_object,
 * ptychographic_methods.py:814-847, applied to the slice update of
 * ptychographic_tomography.py:1115-1119). out_mode 1 writes a float64 volume;
 * 2 adds into a float32 volume (float64 sum rounded once).
 */
int ptycho_volume_expand_update(const float* sliced, const float* sliced_old,
                                int32_t num_slices, int32_t n0, int32_t n1, int32_t n2,
                                void* out, int32_t out_mode, void* stream);

/* volume += addend / divisor, in float32 (ptychographic_tomography.py:1225-1226). */
int ptycho_volume_add_scaled(float* volume, const float* addend, int64_t count, int32_t divisor,
                             void* stream);

/*
 * Volume object constraints: v -= shrinkage (apply_shrinkage), then v = max(v, 0)
 * (positivity), float32 (ptychographic_constraints.py:60-118 and 836-887 with no
 * object mask).
 */
int ptycho_volume_constraints(float* volume, int64_t count, float shrinkage,
                              int32_t apply_shrinkage, int32_t positivity, void* stream);

/*
 * The per-iteration error read-back: copies the device float *error_accum (the
 * sum the batch calls add to) into *value, after the work queued on `stream`
 * has finished, and returns PTYCHO_ERR_NONFINITE when it is NaN or infinite.
 * A batch call makes its error sum NaN when a scan position is not finite (the
 * position is then left out of every patch index and, under position
 * correction, not moved) or when an update produced a NaN or infinite object or
 * probe value; NaN or infinite amplitudes, probes or objects reach the sum
 * through the forward model. Replaces the error read of reconstruct()
 * (singleslice_ptychography.py:929-932), the one synchronisation per iteration.
 */
int ptycho_read_error(const float* error_accum, float* value, void* stream);

/*
 * Instrumentation. When enabled, every launch of the fused per-position kernel
 * is bracketed by CUDA events recorded on its stream; ptycho_kernel_timing()
 * waits for the last one and returns the summed kernel time (ms) and the number
 * of launches since the previous query, then clears the record. No reference
 * counterpart (the reference has no kernels of its own on this path).
 */
int ptycho_enable_kernel_timing(int32_t enable);
int ptycho_kernel_timing(float* total_ms, int32_t* launches);

/*
 * ptycho_gd_batch() for callers that cannot allocate device memory (an
 * acquisition loop with a device-memory budget fixed at start-up, or a host
 * application whose own allocator owns the GPU): same arguments and results
 * without the workspace; the scratch is a fixed 32 MiB array inside the
 * library that each GPU holds from loading the library until exit. Batches
 * needing more scratch than that (ptycho_workspace_bytes) return
 * PTYCHO_ERR_WORKSPACE. The first call on a device looks up the array's
 * address and should come before any stream capture. All calls share the
 * array: calls that can overlap on the GPU must be serialised on one stream.
 * The batch-chaining flags PTYCHO_FLAG_SPECTRUM_READY, PTYCHO_FLAG_PREPARE_SPECTRUM
 * and PTYCHO_FLAG_KEEP_FARFIELD are refused (PTYCHO_ERR_INVALID_ARGUMENT): each
 * call computes its own probe spectrum. No counterpart in the reference (its
 * CuPy path always allocates).
 */
int ptycho_gd_batch_noalloc(const ptycho_geometry* geometry, void* object, void* probe,
                            const float* amplitudes, const int32_t* amplitude_rows,
                            const float* positions_px, const int32_t* position_rows,
                            int32_t batch, float step_size, float normalization_min,
                            int32_t fix_probe, const float* detector_mask,
                            const void* propagators, float* error_accum, void* stream);

/*
 * Kernel schedule for the fused per-position kernel of a given ROI edge length:
 * 0 = library default, 1 = shared-memory Stockham passes (every ROI and
 * variant), 2 = register-resident four-step transform (128 x 128 single-slice
 * gradient descent only; other cases fall back to 1), 3 = shared-memory passes
 * by groups of warps that each own 16 rows / columns, with block-wide barriers
 * only between the axes of a transform (128 x 128: gradient descent of every
 * model, projection sets of one slice and probe, the position correction of
 * single-slice batches; other cases fall back to 1). The default is 3 where it
 * applies, else 1. Process-wide; results agree between schedules to float32
 * rounding. Returns the previous setting (0-3), or -PTYCHO_ERR_INVALID_ARGUMENT
 * for a schedule outside 0-3 (the setting is then unchanged).
 * No reference counterpart (tuning knob of this library's autotuner).
 */
int ptycho_set_kernel_schedule(int32_t roi, int32_t schedule);

/*
 * FP32 throughput probe: `blocks` blocks of 256 threads each run `iters`
 * iterations of 8 independent FMA chains and write one float per thread to
 * `sink` (device, blocks*256 floats). 16 * blocks * 256 * iters flops. Used to
 * measure the FP32 (non-tensor) peak the FFT kernels are judged against.
 */
int ptycho_fp32_fma_probe(int32_t blocks, int32_t iters, float* sink, void* stream);

/*
 * Learned initializer (no counterpart in the reference). A 4-level U-Net with
 * 32 base channels maps a scan's virtual bright-field and centre-of-mass
 * magnitude images to an initial object phase. Weights and activations are
 * bfloat16 (passed as raw 16-bit words), accumulation is float32, and the 3 x 3
 * convolutions are implicit GEMMs on the tensor cores (tcgen05.mma with TMEM
 * accumulators). Every buffer belongs to the caller; no call allocates. Waits
 * inside the tensor-core kernels are bounded: on time-out they set the int
 * error word the call names (err_flag, or the U-Net workspace's own word) and
 * return.
 *
 * ptycho_nn_gemm_bf16: c (m, n) float32 = a (m, k) b (n, k)^T, bf16 row-major
 * operands; n a multiple of 16, k a multiple of 8.
 *
 * ptycho_nn_conv3x3_*: 3 x 3 convolution, stride 1, zero padding 1, NHWC bf16
 * activations (batch, height, width, channels); cin a multiple of 8, cout a
 * multiple of 16, width a multiple of 8. weight (cout, 9, cin) bf16 with the
 * tap index ky * 3 + kx; weight_t (cin, 9, cout) the same values with the
 * channel axes exchanged. forward: y = act(conv(x) + bias) in bf16 (bias may be
 * NULL; relu != 0 applies max(0, .)). backward_data: dx (batch, height, width,
 * cin) float32 = the gradient wrt x for the gradient dy wrt the convolution's
 * output. backward_weight: dweight (cout, 9, cin) and dbias (cout, or NULL)
 * float32, summed over the batch in a fixed order (workspace:
 * ptycho_nn_conv3x3_wgrad_workspace_bytes).
 */
int ptycho_nn_gemm_bf16(const void* a, const void* b, float* c, int32_t m, int32_t n, int32_t k,
                        int32_t* err_flag, void* stream);
int ptycho_nn_conv3x3_forward(const void* x, int32_t batch, int32_t height, int32_t width,
                              int32_t cin, const void* weight, const float* bias, int32_t cout,
                              int32_t relu, void* y, int32_t* err_flag, void* stream);
int ptycho_nn_conv3x3_backward_data(const void* dy, int32_t batch, int32_t height,
                                    int32_t width, int32_t cout, const void* weight_t,
                                    int32_t cin, float* dx, int32_t* err_flag, void* stream);
size_t ptycho_nn_conv3x3_wgrad_workspace_bytes(int32_t batch, int32_t height, int32_t width,
                                               int32_t cin, int32_t cout);
int ptycho_nn_conv3x3_backward_weight(const void* x, const void* dy, int32_t batch,
                                      int32_t height, int32_t width, int32_t cin, int32_t cout,
                                      float* dweight, float* dbias, void* workspace,
                                      size_t workspace_bytes, int32_t* err_flag, void* stream);

/*
 * The U-Net. params: ptycho_nn_unet_param_bytes() bytes (256-byte aligned)
 * holding, per layer, the bf16 weights and their transpose, float32 master
 * weights and biases, their gradients of the last training step and the Adam
 * moments; ptycho_nn_unet_param_offset(layer, field) gives the byte offset of
 * one of them (layers 0..13 the 3 x 3 convolutions, 14 the 1 x 1 head; field 0
 * bf16 weights, 1 bf16 transposed weights, 2 float32 weights, 3 float32 bias,
 * 4 weight gradient, 5 bias gradient) or -1. ptycho_nn_unet_init fills them
 * (He-normal weights from `seed`, zero biases and moments).
 * workspace: ptycho_nn_unet_workspace_bytes(batch, height, width) bytes,
 * 256-byte aligned and zeroed once by the caller (it holds the error word that
 * ptycho_nn_check reads and clears); height and width multiples of 64.
 * input (batch, height, width, 2) float32, output / target / mask (batch,
 * height, width) float32. train_step: forward, loss = sum(mask (out - target)^2)
 * / mask_count (mask NULL = all ones) into *loss (device float), backward, one
 * Adam step (learning_rate, step >= 1 counts the steps for the bias
 * correction; beta 0.9 / 0.999, eps 1e-8).
 */
size_t ptycho_nn_unet_param_bytes(void);
int64_t ptycho_nn_unet_param_offset(int32_t layer, int32_t field);
size_t ptycho_nn_unet_workspace_bytes(int32_t batch, int32_t height, int32_t width);
int ptycho_nn_unet_init(void* params, uint64_t seed, void* stream);
int ptycho_nn_unet_forward(const void* params, const float* input, int32_t batch, int32_t height,
                           int32_t width, float* output, void* workspace, size_t workspace_bytes,
                           void* stream);
int ptycho_nn_unet_train_step(void* params, const float* input, const float* target,
                              const float* mask, float mask_count, int32_t batch, int32_t height,
                              int32_t width, float learning_rate, int32_t step, float* loss,
                              void* workspace, size_t workspace_bytes, void* stream);
/*
 * Training data and inputs of the learned initializer.
 * ptycho_nn_lattice_objects: `count` synthetic objects (object_px square at
 * `sampling` Angstrom per pixel): phase = peak * sum of Gaussian atoms
 * (sigma Angstrom) on a square lattice, params (count, 5) float32 = lattice
 * constant (Angstrom), rotation (rad), lattice offset x, y (Angstrom), unused;
 * phase and phase_blur (the phase blurred by a Gaussian of sigma_blur
 * Angstrom) (count, P, P) float32, object = exp(-0.1 phase) exp(i phase)
 * complex64.
 * ptycho_nn_scan_images: for scan s and position j (128 x 128 detector): the
 * far field of the sub-pixel shifted probe (spectra (scans, 128, 128) complex64,
 * FFT2 of each scan's probe) times the object patch at positions_px (scans, J, 2),
 * its intensities scaled to `dose` counts; bf = counts inside the bright-field
 * disc (radius bf_radius_px), com_x / com_y = centre of mass of the counts in
 * detector pixels, with the Poisson noise of those sums from their normal
 * approximations (keyed by seed, s and j); target = `phase` (the caller passes
 * the blurred phase) at the position, bilinear; all (scans, J) float32.
 * ptycho_nn_virtual_images: the same bright-field sum and centre of mass of
 * the intensities amplitudes^2 of `count` corner-centred (sx, sy) patterns.
 */
int ptycho_nn_lattice_objects(int32_t count, int32_t object_px, float sampling,
                              const float* params, float sigma, float peak, float sigma_blur,
                              float* phase, float* phase_blur, void* object, void* stream);
int ptycho_nn_scan_images(int32_t scans, int32_t positions, int32_t object_px,
                          const void* spectra, const void* objects, const float* phase,
                          const float* positions_px, float dose, float bf_radius_px,
                          uint64_t seed, float* bf, float* com_x, float* com_y, float* target,
                          void* stream);
int ptycho_nn_virtual_images(const float* amplitudes, int32_t count, int32_t sx, int32_t sy,
                             float bf_radius_px, float* bf, float* com_x, float* com_y,
                             void* stream);

/* Waits for `stream`, then returns PTYCHO_ERR_CUDA (and clears the word) if a
 * tensor-core wait of the U-Net kernels timed out since the last check. */
int ptycho_nn_check(void* workspace, int32_t batch, int32_t height, int32_t width, void* stream);
const char* ptycho_nn_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PTYCHO_GB300_H */
