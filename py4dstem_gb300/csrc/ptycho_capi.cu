// extern "C" entry points of libptycho_gb300.so (declared in include/ptycho_gb300.h).
// Validates arguments, carves the caller's workspace and launches the kernels of
// ptycho_position.cuh (instantiated per region-of-interest size) and ptycho_reduce.cu
// on the caller's stream.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/ptycho_gb300.h"
#include "ptycho_internal.h"

namespace pty {
namespace {

thread_local char g_last_error[512] = "";

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(PTYCHO_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// ---- position-kernel timing: pairs of events recorded around each launch
std::mutex g_timing_mu;
bool g_timing_on = false;
std::vector<cudaEvent_t> g_ev_pool;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_ev_pairs;
cudaEvent_t g_ev_pending = nullptr;

cudaEvent_t take_event() {
  if (!g_ev_pool.empty()) {
    cudaEvent_t e = g_ev_pool.back();
    g_ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

int detector_x(const ptycho_geometry* g) { return g->detector_x ? g->detector_x : g->roi_x; }
int detector_y(const ptycho_geometry* g) { return g->detector_y ? g->detector_y : g->roi_y; }

int check_geometry(const ptycho_geometry* g) {
  if (!g) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "geometry is null");
  if ((g->flags & ~(PTYCHO_FLAG_MIXED_STATE | PTYCHO_FLAG_KEEP_FARFIELD |
                    PTYCHO_FLAG_SPECTRUM_READY | PTYCHO_FLAG_PREPARE_SPECTRUM)) != 0)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "unknown bits in geometry.flags (0x%x)", g->flags);
  if (g->num_slices < 1 || g->num_probes < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "num_slices and num_probes must be >= 1");
  if (g->num_probes > 16) return fail(PTYCHO_ERR_UNSUPPORTED, "at most 16 probe modes");
  if (!roi_supported(g->roi_x, g->roi_y))
    return fail(PTYCHO_ERR_UNSUPPORTED,
                "ROI %dx%d has no kernel (supported: square 32, 48, 64, 96, 128, 256 "
                "and 96 x 128, 128 x 96)",
                g->roi_x, g->roi_y);
  if ((g->detector_x == 0) != (g->detector_y == 0) || g->detector_x < 0 ||
      g->detector_y < 0 || (g->detector_x != 0 && (g->detector_x < 2 || g->detector_y < 2)))
    return fail(PTYCHO_ERR_INVALID_ARGUMENT,
                "detector_x and detector_y must both be 0 (the ROI shape) or both >= 2 "
                "(got %d x %d)", g->detector_x, g->detector_y);
  if (detector_x(g) > 4096 || detector_y(g) > 4096)
    return fail(PTYCHO_ERR_UNSUPPORTED, "detector %d x %d larger than 4096 x 4096",
                detector_x(g), detector_y(g));
  if ((staged_roi(g->roi_x, g->roi_y) || detector_x(g) != g->roi_x ||
       detector_y(g) != g->roi_y) &&
      (g->flags & PTYCHO_FLAG_KEEP_FARFIELD) != 0)
    return fail(PTYCHO_ERR_UNSUPPORTED,
                "PTYCHO_FLAG_KEEP_FARFIELD (position correction) is not available for a %d x %d "
                "ROI or a resampled far field", g->roi_x, g->roi_y);
  if (g->object_x < g->roi_x || g->object_y < g->roi_y)
    return fail(PTYCHO_ERR_UNSUPPORTED, "object %dx%d smaller than ROI %dx%d", g->object_x,
                g->object_y, g->roi_x, g->roi_y);
  if (g->object_is_potential != 0 && g->object_is_potential != 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object_is_potential must be 0 or 1");
  return PTYCHO_OK;
}

std::mutex g_smem_mu;
std::map<std::pair<int, const void*>, int> g_smem_limits;  // (device, kernel) -> bytes set

}  // namespace

cudaError_t ensure_smem_limit(const void* fn, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_smem_mu);
  auto it = g_smem_limits.find({dev, fn});
  if (it != g_smem_limits.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  g_smem_limits[{dev, fn}] = bytes;
  return cudaSuccess;
}

Workspace workspace_layout(int Sx, int Sy, int Px, int Py, int T, int M, int B,
                           bool keep_farfield, int Ax, int Ay) {
  Workspace w{};
  const size_t N = (size_t)Sx * Sy;
  const bool resample = Ax != Sx || Ay != Sy;
  const bool staged = staged_roi(Sx, Sy) || resample;
  const size_t Nd = (size_t)Ax * Ay;
  const size_t chunks = ((resample ? Nd : N) + 2047) / 2048;
  const size_t P = (size_t)Px * Py;
  const size_t ntiles = (size_t)((Px + kTile - 1) / kTile) * ((Py + kTile - 1) / kTile);
  const size_t nb = (N + kReduceThreads - 1) / kReduceThreads;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  w.probe_spec = take(sizeof(float2) * M * N);
  w.tw = take(sizeof(float2) * (Sx + Sy));
  w.st_obj = take(sizeof(float2) * T * B * N);
  w.st_nobj = take(sizeof(float) * T * B * N);
  w.st_probe = take(sizeof(float2) * B * M * N);
  w.st_nprobe = take(sizeof(float) * B * N);
  const bool mixed_ms = T > 1 && M > 1;
  w.scratch_f =
      take(T == 1 || keep_farfield || mixed_ms || staged ? sizeof(float2) * B * M * N : 0);
  w.st_pm = take(mixed_ms ? sizeof(float2) * T * B * M * N : 0);
  w.pos_round = take(sizeof(int2) * B);
  w.err = take(sizeof(float) * B);
  w.err_part = take(staged ? sizeof(float) * B * chunks : 0);
  w.det_f = take(resample ? sizeof(float2) * B * M * Nd : 0);
  w.obj_grad = take(sizeof(float2) * T * P);
  w.obj_nrm = take(sizeof(float) * T * P);
  w.tile_max = take(sizeof(float) * T * ntiles);
  w.probe_part = take(sizeof(float2) * kProbeChunks * M * N);
  w.probe_npart = take(sizeof(float) * kProbeChunks * N);
  w.probe_bmax = take(sizeof(float) * nb);
  w.probe_grad = take(sizeof(float2) * M * N);
  w.probe_nrm = take(sizeof(float) * N);
  w.com = take(sizeof(double) * 4);
  w.red = take(sizeof(double) * 1024);
  w.total = off;
  return w;
}

void bind_workspace(BatchArgs& a, void* base, const Workspace& w) {
  char* p = static_cast<char*>(base);
  a.probe_spec = reinterpret_cast<float2*>(p + w.probe_spec);
  a.tw = reinterpret_cast<float2*>(p + w.tw);
  a.st_obj = reinterpret_cast<float2*>(p + w.st_obj);
  a.st_nobj = reinterpret_cast<float*>(p + w.st_nobj);
  a.st_probe = reinterpret_cast<float2*>(p + w.st_probe);
  a.st_nprobe = reinterpret_cast<float*>(p + w.st_nprobe);
  a.scratch_f = reinterpret_cast<float2*>(p + w.scratch_f);
  a.st_pm = reinterpret_cast<float2*>(p + w.st_pm);
  a.pos_round = reinterpret_cast<int2*>(p + w.pos_round);
  a.err = reinterpret_cast<float*>(p + w.err);
  a.err_part = reinterpret_cast<float*>(p + w.err_part);
  a.det_f = reinterpret_cast<float2*>(p + w.det_f);
  a.obj_grad = reinterpret_cast<float2*>(p + w.obj_grad);
  a.obj_nrm = reinterpret_cast<float*>(p + w.obj_nrm);
  a.tile_max = reinterpret_cast<float*>(p + w.tile_max);
  a.probe_part = reinterpret_cast<float2*>(p + w.probe_part);
  a.probe_npart = reinterpret_cast<float*>(p + w.probe_npart);
  a.probe_bmax = reinterpret_cast<float*>(p + w.probe_bmax);
  a.probe_grad = reinterpret_cast<float2*>(p + w.probe_grad);
  a.probe_nrm = reinterpret_cast<float*>(p + w.probe_nrm);
  a.com = reinterpret_cast<double*>(p + w.com);
  a.red = reinterpret_cast<float*>(p + w.red);
}

namespace {

int prepare(const ptycho_geometry* g, int32_t batch, void* workspace, size_t workspace_bytes,
            BatchArgs& a) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (batch < 1) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "batch must be >= 1 (got %d)", batch);
  if (!workspace) return fail(PTYCHO_ERR_WORKSPACE, "workspace is null");
  if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
    return fail(PTYCHO_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  const Workspace w = workspace_layout(g->roi_x, g->roi_y, g->object_x, g->object_y,
                                       g->num_slices, g->num_probes, batch,
                                       (g->flags & PTYCHO_FLAG_KEEP_FARFIELD) != 0,
                                       detector_x(g), detector_y(g));
  if (workspace_bytes < w.total)
    return fail(PTYCHO_ERR_WORKSPACE, "workspace of %zu bytes is smaller than the %zu needed",
                workspace_bytes, w.total);
  std::memset(&a, 0, sizeof(a));
  a.Sx = g->roi_x;
  a.Sy = g->roi_y;
  a.Ax = detector_x(g);
  a.Ay = detector_y(g);
  a.resample = a.Ax != a.Sx || a.Ay != a.Sy ? 1 : 0;
  a.Px = g->object_x;
  a.Py = g->object_y;
  a.T = g->num_slices;
  a.M = g->num_probes;
  a.potential = g->object_is_potential;
  a.B = batch;
  bind_workspace(a, workspace, w);
  return PTYCHO_OK;
}

}  // namespace

void timing_before(cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_timing_mu);
  if (!g_timing_on) return;
  g_ev_pending = take_event();
  cudaEventRecord(g_ev_pending, s);
}

void timing_after(cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_timing_mu);
  if (!g_timing_on || !g_ev_pending) return;
  cudaEvent_t stop = take_event();
  cudaEventRecord(stop, s);
  g_ev_pairs.emplace_back(g_ev_pending, stop);
  g_ev_pending = nullptr;
}

}  // namespace pty

using namespace pty;

extern "C" {

int ptycho_abi_version(void) { return PTYCHO_ABI_VERSION; }

const char* ptycho_last_error(void) { return g_last_error; }

int ptycho_roi_supported(int32_t roi_x, int32_t roi_y) { return roi_supported(roi_x, roi_y) ? 1 : 0; }

int ptycho_geometry_supported(const ptycho_geometry* g) { return check_geometry(g); }

size_t ptycho_workspace_bytes(const ptycho_geometry* g, int32_t max_batch) {
  if (!g || max_batch < 1) return 0;
  if (check_geometry(g) != PTYCHO_OK) return 0;
  return workspace_layout(g->roi_x, g->roi_y, g->object_x, g->object_y, g->num_slices,
                          g->num_probes, max_batch, (g->flags & PTYCHO_FLAG_KEEP_FARFIELD) != 0,
                          detector_x(g), detector_y(g))
      .total;
}

static int run_batch(const ptycho_geometry* g, void* object, void* probe,
                     const float* amplitudes, const int32_t* amplitude_rows,
                     const float* positions_px, const int32_t* position_rows, int32_t batch,
                     const float* detector_mask, const void* propagators, float* error_accum,
                     void* workspace, size_t workspace_bytes, void* stream, BatchArgs& a) {
  if (!object || !probe || !amplitudes || !positions_px || !error_accum)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object, probe, amplitudes, positions and "
                                             "error_accum must be non-null");
  if (g && g->num_slices > 1 && !propagators)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "multislice needs propagators");
  a.object = object;
  a.probe = static_cast<float2*>(probe);
  a.amplitudes = amplitudes;
  a.amp_rows = amplitude_rows;
  a.positions = positions_px;
  a.pos_rows = position_rows;
  a.det_mask = detector_mask;
  a.props = static_cast<const float2*>(propagators);
  a.error_accum = error_accum;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (!(g->flags & PTYCHO_FLAG_SPECTRUM_READY)) e = launch_probe_spectrum(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "probe spectrum kernel");
  a.prepare_spectrum = (g->flags & PTYCHO_FLAG_PREPARE_SPECTRUM) && !a.fix_probe ? 1 : 0;
  a.staging_t = !staged_batch(a) && position_v2_eligible(a) ? 1 : 0;
  // the plain single-slice GD instantiation of the position kernel stages no
  // |O|^2 terms; the probe-side reduction gathers them from the object
  a.nprobe_from_object = !a.staging_t && !a.projection && !a.forward_only &&
                                 !a.keep_farfield && !a.exact_probe_grad && a.T == 1 &&
                                 a.M == 1 && !a.mixed_formula
                             ? 1
                             : 0;
  e = a.staging_t ? launch_position_v2(a, s) : launch_position_kernel(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "position kernel");
  e = launch_reduce_and_update(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "reduce/update kernels");
  return PTYCHO_OK;
}

int ptycho_gd_batch(const ptycho_geometry* g, void* object, void* probe,
                    const float* amplitudes, const int32_t* amplitude_rows,
                    const float* positions_px, const int32_t* position_rows, int32_t batch,
                    float step_size, float normalization_min, int32_t fix_probe,
                    const float* detector_mask, const void* propagators, float* error_accum,
                    void* workspace, size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  a.step = step_size;
  a.norm_min = normalization_min;
  a.fix_probe = fix_probe ? 1 : 0;
  a.mixed_formula = (g->num_probes > 1 || (g->flags & PTYCHO_FLAG_MIXED_STATE)) ? 1 : 0;
  a.keep_farfield = (g->flags & PTYCHO_FLAG_KEEP_FARFIELD) ? 1 : 0;
  return run_batch(g, object, probe, amplitudes, amplitude_rows, positions_px, position_rows,
                   batch, detector_mask, propagators, error_accum, workspace, workspace_bytes,
                   stream, a);
}

int ptycho_projection_batch(const ptycho_geometry* g, void* object, void* probe,
                            const float* amplitudes, const int32_t* amplitude_rows,
                            const float* positions_px, const int32_t* position_rows,
                            int32_t batch, float projection_a, float projection_b,
                            float projection_c, float normalization_min, int32_t fix_probe,
                            void* exit_waves, int32_t exit_waves_valid, const void* propagators,
                            float* error_accum, void* workspace, size_t workspace_bytes,
                            void* stream) {
  BatchArgs a;
  int st = prepare(g, batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!exit_waves) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "exit_waves must be non-null");
  if (staged_batch(a))
    return fail(PTYCHO_ERR_UNSUPPORTED, "projection sets are not available for a %d x %d ROI "
                "or a resampled far field", g->roi_x, g->roi_y);
  a.projection = 1;
  a.keep_farfield = (g->flags & PTYCHO_FLAG_KEEP_FARFIELD) ? 1 : 0;
  a.pa = projection_a;
  a.pb = projection_b;
  a.pc = projection_c;
  a.norm_min = normalization_min;
  a.fix_probe = fix_probe ? 1 : 0;
  a.exit_waves = static_cast<float2*>(exit_waves);
  a.ew_valid = exit_waves_valid ? 1 : 0;
  a.mixed_formula = (g->num_probes > 1 || (g->flags & PTYCHO_FLAG_MIXED_STATE)) ? 1 : 0;
  return run_batch(g, object, probe, amplitudes, amplitude_rows, positions_px, position_rows,
                   batch, nullptr, propagators, error_accum, workspace, workspace_bytes, stream,
                   a);
}

int ptycho_position_correction(const ptycho_geometry* g, const void* object,
                               const void* probe, const void* propagators,
                               const float* amplitudes, const int32_t* amplitude_rows,
                               float* positions_px, const float* positions_initial,
                               const int32_t* position_rows, int32_t batch, float step_size,
                               double max_update_px, double max_total_px, void* workspace,
                               size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!(g->flags & PTYCHO_FLAG_KEEP_FARFIELD))
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "position correction needs the far fields of a "
                                             "batch run with PTYCHO_FLAG_KEEP_FARFIELD");

  if (!object || !amplitudes || !positions_px || !positions_initial)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object, amplitudes, positions_px and "
                                             "positions_initial must be non-null");
  if (g->num_slices > 1 && (!probe || !propagators))
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "multislice position correction needs the probe "
                                             "and the propagators");
  a.object = const_cast<void*>(object);
  a.amplitudes = amplitudes;
  a.amp_rows = amplitude_rows;
  a.positions = positions_px;
  a.positions_rw = positions_px;
  a.positions_initial = positions_initial;
  a.pos_rows = position_rows;
  a.pc_step = step_size;
  a.pc_max_update = max_update_px;
  a.pc_max_total = max_total_px;
  a.mixed_formula = (g->num_probes > 1 || (g->flags & PTYCHO_FLAG_MIXED_STATE)) ? 1 : 0;
  a.probe = static_cast<float2*>(const_cast<void*>(probe));
  a.props = static_cast<const float2*>(propagators);
  cudaError_t e = launch_position_correction(a, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "position correction kernel");
  return PTYCHO_OK;
}

int ptycho_self_consistency_errors(const ptycho_geometry* g, const void* object,
                                   const void* probe, const float* amplitudes,
                                   const int32_t* amplitude_rows, const float* positions_px,
                                   const int32_t* position_rows, int32_t batch,
                                   const void* propagators, float* errors, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!object || !probe || !amplitudes || !positions_px || !errors)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object, probe, amplitudes, positions and errors "
                                             "must be non-null");
  if (g->num_slices > 1 && !propagators)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "multislice needs propagators");
  a.forward_only = 1;
  a.mixed_formula = (g->num_probes > 1 || (g->flags & PTYCHO_FLAG_MIXED_STATE)) ? 1 : 0;
  a.object = const_cast<void*>(object);
  a.probe = static_cast<float2*>(const_cast<void*>(probe));
  a.amplitudes = amplitudes;
  a.amp_rows = amplitude_rows;
  a.positions = positions_px;
  a.pos_rows = position_rows;
  a.props = static_cast<const float2*>(propagators);
  a.err = errors;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = launch_probe_spectrum(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "probe spectrum kernel");
  e = launch_position_kernel(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "position kernel (forward only)");
  return PTYCHO_OK;
}

int ptycho_gd_gradient(const ptycho_geometry* g, const void* object, const void* probe,
                       const float* amplitudes, const int32_t* amplitude_rows,
                       const float* positions_px, const int32_t* position_rows, int32_t batch,
                       const float* detector_mask, const void* propagators, void* object_grad,
                       void* probe_grad, float* loss, void* workspace, size_t workspace_bytes,
                       void* stream) {
  BatchArgs a;
  int st = prepare(g, batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!object || !probe || !amplitudes || !positions_px || !object_grad || !loss)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object, probe, amplitudes, positions, object_grad "
                                             "and loss must be non-null");
  if (g->num_slices > 1 && !propagators)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "multislice needs propagators");
  if (probe_grad && staged_batch(a))
    return fail(PTYCHO_ERR_UNSUPPORTED, "the probe gradient is not available for a %d x %d ROI "
                "or a resampled far field (pass probe_grad = null for the object gradient)",
                g->roi_x, g->roi_y);
  a.mixed_formula = (g->num_probes > 1 || (g->flags & PTYCHO_FLAG_MIXED_STATE)) ? 1 : 0;
  a.object = const_cast<void*>(object);
  a.probe = static_cast<float2*>(const_cast<void*>(probe));
  a.amplitudes = amplitudes;
  a.amp_rows = amplitude_rows;
  a.positions = positions_px;
  a.pos_rows = position_rows;
  a.det_mask = detector_mask;
  a.props = static_cast<const float2*>(propagators);
  a.exact_probe_grad = probe_grad ? 1 : 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = launch_probe_spectrum(a, s);
  if (e != cudaSuccess) return cuda_fail(e, "probe spectrum kernel");
  e = launch_position_kernel(a, s);  // natural staging order (the shared-memory schedule)
  if (e != cudaSuccess) return cuda_fail(e, "position kernel");
  e = launch_gradient(a, object_grad, static_cast<float2*>(probe_grad), loss, s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient kernels");
  return PTYCHO_OK;
}

int ptycho_object_constraints(const ptycho_geometry* g, void* object, const uint8_t* mask,
                              float shrinkage_rad, int32_t apply_shrinkage, int32_t pure_phase,
                              int32_t positivity, void* workspace, size_t workspace_bytes,
                              void* stream) {
  BatchArgs a;
  int st = prepare(g, 1, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!object) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object is null");
  a.object = object;
  cudaError_t e = launch_object_constraints(a, mask, shrinkage_rad, apply_shrinkage, pure_phase,
                                            positivity, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "object constraints");
  return PTYCHO_OK;
}

int ptycho_probe_com_constraint(const ptycho_geometry* g, void* probe, void* workspace,
                                size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, 1, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!probe) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe is null");
  a.probe = static_cast<float2*>(probe);
  cudaError_t e = launch_probe_com(a, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe CoM constraint");
  return PTYCHO_OK;
}

int ptycho_mapped_host_pointer(const void* host, size_t bytes, void** device) {
  if (!device) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "device must be non-null");
  *device = nullptr;
  if (!host || bytes == 0) return PTYCHO_OK;
  cudaPointerAttributes first, last;
  if (cudaPointerGetAttributes(&first, host) != cudaSuccess) {
    cudaGetLastError();  // no device or an unknown pointer: not mapped
    return PTYCHO_OK;
  }
  if (first.type != cudaMemoryTypeHost || first.devicePointer == nullptr) return PTYCHO_OK;
  // the whole range must lie in one page-locked, mapped allocation
  const char* end = static_cast<const char*>(host) + bytes - 1;
  if (cudaPointerGetAttributes(&last, end) != cudaSuccess) {
    cudaGetLastError();
    return PTYCHO_OK;
  }
  if (last.type != cudaMemoryTypeHost || last.devicePointer == nullptr ||
      static_cast<const char*>(last.devicePointer) !=
          static_cast<const char*>(first.devicePointer) + bytes - 1)
    return PTYCHO_OK;
  *device = first.devicePointer;
  return PTYCHO_OK;
}

int ptycho_prepare_stream(void* stream) {
  cudaError_t e = prepare_stream(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "helper stream");
  return PTYCHO_OK;
}

int ptycho_set_kernel_schedule(int32_t roi, int32_t schedule) {
  if (schedule < 0 || schedule > 3) {
    // (negative: a previous setting is never negative, a status could be one)
    fail(PTYCHO_ERR_INVALID_ARGUMENT, "schedule must be 0, 1, 2 or 3 (got %d)", schedule);
    return -PTYCHO_ERR_INVALID_ARGUMENT;
  }
  return set_schedule(roi, schedule);
}

int ptycho_read_error(const float* error_accum, float* value, void* stream) {
  if (!error_accum || !value)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "error_accum and value must be non-null");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float v = 0.0f;
  cudaError_t e = cudaMemcpyAsync(&v, error_accum, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "error read-back");
  *value = v;
  if (!std::isfinite(v))
    return fail(PTYCHO_ERR_NONFINITE,
                "the error sum is %s: a scan position, amplitude, probe or object value is "
                "NaN or infinite, or an update overflowed",
                std::isnan(v) ? "NaN" : "infinite");
  return PTYCHO_OK;
}

int ptycho_enable_kernel_timing(int32_t enable) {
  std::lock_guard<std::mutex> lk(g_timing_mu);
  g_timing_on = enable != 0;
  return PTYCHO_OK;
}

int ptycho_kernel_timing(float* total_ms, int32_t* launches) {
  if (!total_ms || !launches)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "total_ms and launches must be non-null");
  std::lock_guard<std::mutex> lk(g_timing_mu);
  float sum = 0.f;
  int n = 0;
  for (auto& pr : g_ev_pairs) {
    cudaError_t e = cudaEventSynchronize(pr.second);
    if (e != cudaSuccess) return cuda_fail(e, "timing event");
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, pr.first, pr.second);
    if (e != cudaSuccess) return cuda_fail(e, "timing elapsed");
    sum += ms;
    ++n;
    g_ev_pool.push_back(pr.first);
    g_ev_pool.push_back(pr.second);
  }
  g_ev_pairs.clear();
  *total_ms = sum;
  *launches = n;
  return PTYCHO_OK;
}

int ptycho_fp32_fma_probe(int32_t blocks, int32_t iters, float* sink, void* stream) {
  if (blocks < 1 || iters < 1 || !sink)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "blocks, iters >= 1 and sink non-null required");
  cudaError_t e = launch_fma_probe(blocks, iters, sink, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "fma probe");
  return PTYCHO_OK;
}

int ptycho_probe_gram(const ptycho_geometry* g, const void* probe, void* gram, void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!probe || !gram) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe and gram must be non-null");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Sx = g->roi_x;
  a.Sy = g->roi_y;
  a.M = g->num_probes;
  cudaError_t e = launch_probe_gram(a, static_cast<const float2*>(probe),
                                    static_cast<float2*>(gram), static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe Gram matrix");
  return PTYCHO_OK;
}

int ptycho_probe_orthogonalize(const ptycho_geometry* g, void* probe, void* workspace,
                               size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, 1, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!probe) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe is null");
  a.probe = static_cast<float2*>(probe);
  // scratch: the probe-gradient rows (M x N) and the constraint scratch (Gram, coefficients)
  float2* gram = reinterpret_cast<float2*>(a.red);
  float2* coeffs = gram + 16 * 16;
  cudaError_t e = launch_probe_orthogonalize(a, a.probe_grad, gram, coeffs,
                                             static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe orthogonalisation");
  return PTYCHO_OK;
}

int ptycho_probe_mix(const ptycho_geometry* g, const void* probe_in, const void* coeffs,
                     void* probe_out, void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!probe_in || !coeffs || !probe_out)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe_in, coeffs and probe_out must be non-null");
  if (probe_in == probe_out) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe_out aliases probe_in");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Sx = g->roi_x;
  a.Sy = g->roi_y;
  a.M = g->num_probes;
  cudaError_t e = launch_probe_mix(a, static_cast<const float2*>(probe_in),
                                   static_cast<const float2*>(coeffs),
                                   static_cast<float2*>(probe_out),
                                   static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe mix");
  return PTYCHO_OK;
}

// ------------------------------------------------------- optional constraints
int ptycho_object_identical_slices(const ptycho_geometry* g, void* object, void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!object) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object must be non-null");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Px = g->object_x;
  a.Py = g->object_y;
  a.T = g->num_slices;
  a.potential = g->object_is_potential;
  a.object = object;
  cudaError_t e = launch_identical_slices(a, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "identical-slices kernel");
  return PTYCHO_OK;
}

int ptycho_object_gaussian_constraint(const ptycho_geometry* g, void* object,
                                      const double* weights, int32_t radius,
                                      int32_t pure_phase, void* scratch, void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!object || !weights || !scratch)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "object, weights and scratch must be non-null");
  if (radius < 0) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "radius must be >= 0");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Px = g->object_x;
  a.Py = g->object_y;
  a.T = g->num_slices;
  a.potential = g->object_is_potential;
  a.object = object;
  cudaError_t e = launch_object_gaussian(a, weights, radius, pure_phase ? 1 : 0,
                                         static_cast<float*>(scratch),
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "object Gaussian kernels");
  return PTYCHO_OK;
}

int ptycho_probe_aperture_constraint(const ptycho_geometry* g, void* probe,
                                     const float* aperture, void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!probe || !aperture)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe and aperture must be non-null");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Sx = g->roi_x;
  a.Sy = g->roi_y;
  a.M = g->num_probes;
  a.probe = static_cast<float2*>(probe);
  a.aperture = aperture;
  cudaError_t e = launch_probe_aperture(a, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe aperture kernel");
  return PTYCHO_OK;
}

int ptycho_probe_amplitude_constraint(const ptycho_geometry* g, void* probe, const float* mask,
                                      void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (!probe || !mask) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe and mask must be non-null");
  BatchArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Sx = g->roi_x;
  a.Sy = g->roi_y;
  a.M = g->num_probes;
  a.probe = static_cast<float2*>(probe);
  cudaError_t e = launch_probe_amplitude(a, mask, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe amplitude kernel");
  return PTYCHO_OK;
}

// ----------------------------------------------------------------- preprocess
int ptycho_pattern_com(const float* intensities, int32_t num_patterns, int32_t qx, int32_t qy,
                       const void* mask, int32_t mask_mode, void* com_x, void* com_y,
                       void* stream) {
  if (!intensities || !com_x || !com_y)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "intensities, com_x and com_y must be non-null");
  if (num_patterns < 0 || qx < 1 || qy < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad pattern count or shape (%d, %d x %d)",
                num_patterns, qx, qy);
  if (mask_mode < 0 || mask_mode > 3 || (mask_mode != 0 && !mask))
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "mask_mode %d needs %s", mask_mode,
                mask_mode < 0 || mask_mode > 3 ? "a value in 0..3" : "a mask");
  if (num_patterns == 0) return PTYCHO_OK;
  cudaError_t e = launch_pattern_com(intensities, num_patterns, qx, qy, mask, mask_mode, com_x,
                                     com_y, static_cast<cudaStream_t>(stream));
  if (e == cudaErrorInvalidValue)
    return fail(PTYCHO_ERR_UNSUPPORTED, "%d x %d patterns do not fit one block's shared memory",
                qx, qy);
  if (e != cudaSuccess) return cuda_fail(e, "pattern centre-of-mass kernel");
  return PTYCHO_OK;
}

int ptycho_rotation_search(const void* com_x, const void* com_y, int32_t com_is_double,
                           int32_t scan_x, int32_t scan_y, const float* cos_angles,
                           const float* sin_angles, int32_t num_angles,
                           int32_t maximize_divergence, void* values, void* stream) {
  if (!com_x || !com_y || !cos_angles || !sin_angles || !values)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "null pointer argument");
  if (scan_x < 3 || scan_y < 3 || num_angles < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT,
                "the rotation search needs a scan of at least 3 x 3 and one angle "
                "(got %d x %d, %d angles)", scan_x, scan_y, num_angles);
  cudaError_t e = launch_rotation_search(com_x, com_y, scan_x, scan_y, cos_angles, sin_angles,
                                         num_angles, maximize_divergence ? 1 : 0,
                                         com_is_double ? 1 : 0, values,
                                         static_cast<cudaStream_t>(stream));
  if (e == cudaErrorInvalidValue)
    return fail(PTYCHO_ERR_UNSUPPORTED, "a %d x %d scan is too large for the rotation search",
                scan_x, scan_y);
  if (e != cudaSuccess) return cuda_fail(e, "rotation search kernel");
  return PTYCHO_OK;
}

int ptycho_normalize_patterns(const float* intensities, int32_t qx, int32_t qy,
                              const int32_t* rows, int32_t num_out, const float* com_fitted_x,
                              const float* com_fitted_y, int32_t crop_w, float* amplitudes,
                              float* pattern_sums, void* stream) {
  if (!intensities || !com_fitted_x || !com_fitted_y || !amplitudes || !pattern_sums)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "null pointer argument");
  if (num_out < 0 || qx < 1 || qy < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad pattern count or shape (%d, %d x %d)",
                num_out, qx, qy);
  if (crop_w < 0 || 2 * crop_w > qx || 2 * crop_w > qy)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "crop width %d does not fit %d x %d patterns",
                crop_w, qx, qy);
  if (num_out == 0) return PTYCHO_OK;
  cudaError_t e = launch_pattern_normalize(intensities, qx, qy, rows, num_out, com_fitted_x,
                                           com_fitted_y, crop_w, amplitudes, pattern_sums,
                                           static_cast<cudaStream_t>(stream));
  if (e == cudaErrorInvalidValue)
    return fail(PTYCHO_ERR_UNSUPPORTED, "%d x %d patterns do not fit one block's shared memory",
                qx, qy);
  if (e != cudaSuccess) return cuda_fail(e, "pattern normalisation kernel");
  return PTYCHO_OK;
}

int ptycho_gather_patterns(const float* patterns, int32_t num_patterns, int64_t pattern_size,
                           const int32_t* rows, int32_t num_out, float* out, void* stream) {
  if (num_out < 0 || num_patterns < 0 || pattern_size < 1 || pattern_size > (int64_t)1 << 28)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad counts (%d of %d patterns of %lld values)",
                num_out, num_patterns, (long long)pattern_size);
  if (num_out == 0) return PTYCHO_OK;
  if (!patterns || !out) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "null pointer argument");
  if (!rows && num_out > num_patterns)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "%d rows requested of %d patterns", num_out,
                num_patterns);
  cudaError_t e = launch_gather_patterns(patterns, rows, num_out, num_patterns,
                                         (int)pattern_size, out, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "pattern gather kernel");
  return PTYCHO_OK;
}

int ptycho_probe_overlap(const ptycho_geometry* g, const void* probe, const float* positions_px,
                         int32_t num_positions, int32_t max_batch, float* overlap,
                         void* workspace, size_t workspace_bytes, void* stream) {
  BatchArgs a;
  int st = prepare(g, max_batch, workspace, workspace_bytes, a);
  if (st != PTYCHO_OK) return st;
  if (!probe || !positions_px || !overlap)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "probe, positions_px and overlap must be non-null");
  if (num_positions < 0)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "num_positions must be >= 0 (got %d)", num_positions);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t P = (size_t)g->object_x * g->object_y;
  cudaError_t e = cudaMemsetAsync(overlap, 0, sizeof(float) * P, s);
  if (e != cudaSuccess) return cuda_fail(e, "overlap clear");
  if (num_positions == 0) return PTYCHO_OK;
  a.probe = static_cast<float2*>(const_cast<void*>(probe));
  a.M = 1;
  a.T = 1;
  a.nobj_only = 1;
  if ((e = launch_probe_spectrum(a, s)) != cudaSuccess) return cuda_fail(e, "probe spectrum");
  // near-equal batches, the larger ones first (utils.py:539-589)
  const int nb = (num_positions + max_batch - 1) / max_batch;
  const int base = num_positions / nb, extra = num_positions % nb;
  int start = 0;
  for (int k = 0; k < nb; ++k) {
    const int size = base + (k < extra ? 1 : 0);
    a.positions = positions_px + 2 * (size_t)start;
    a.B = size;
    if ((e = launch_probe_intensity(a, s)) != cudaSuccess) return cuda_fail(e, "probe intensity");
    if ((e = launch_overlap_accumulate(a, overlap, s)) != cudaSuccess)
      return cuda_fail(e, "overlap accumulation");
    start += size;
  }
  return PTYCHO_OK;
}

// ---- tomography volume operations (ptycho_volume.cu)

int ptycho_volume_rotate(const void* volume, int32_t volume_is_double, void* out,
                         int32_t out_mode, int32_t n0, int32_t n1, int32_t n2,
                         const double* matrix, const double* offset, void* scratch,
                         size_t scratch_bytes, void* stream) {
  if (!volume || !out || !matrix || !offset || !scratch)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT,
                "volume, out, matrix, offset and scratch must be non-null");
  if (n0 < 1 || n1 < 1 || n2 < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad volume shape (%d, %d, %d)", n0, n1, n2);
  if (volume_is_double != 0 && volume_is_double != 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "volume_is_double must be 0 or 1");
  if (out_mode < 0 || out_mode > 2)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "out_mode must be 0, 1 or 2 (got %d)", out_mode);
  const size_t need = (size_t)n0 * n1 * n2 * sizeof(double);
  if (scratch_bytes < need)
    return fail(PTYCHO_ERR_WORKSPACE, "scratch of %zu bytes is smaller than the %zu needed",
                scratch_bytes, need);
  if (reinterpret_cast<uintptr_t>(scratch) % 8 != 0)
    return fail(PTYCHO_ERR_WORKSPACE, "scratch must be 8-byte aligned");
  cudaError_t e = launch_volume_rotate(volume, volume_is_double, out, out_mode, n0, n1, n2,
                                       matrix, offset, static_cast<double*>(scratch),
                                       static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "volume rotation kernels");
  return PTYCHO_OK;
}

int ptycho_volume_project(const float* volume, int32_t n0, int32_t n1, int32_t n2,
                          int32_t num_slices, float* sliced, void* stream) {
  if (!volume || !sliced)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "volume and sliced must be non-null");
  if (n0 < 1 || n1 < 1 || n2 < 1 || num_slices < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad volume shape (%d, %d, %d) or slice count %d",
                n0, n1, n2, num_slices);
  cudaError_t e = launch_volume_project(volume, n0, (size_t)n1 * n2, num_slices, sliced,
                                        static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "volume projection kernel");
  return PTYCHO_OK;
}

int ptycho_volume_expand_update(const float* sliced, const float* sliced_old,
                                int32_t num_slices, int32_t n0, int32_t n1, int32_t n2,
                                void* out, int32_t out_mode, void* stream) {
  if (!sliced || !sliced_old || !out)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "sliced, sliced_old and out must be non-null");
  if (n0 < 1 || n1 < 1 || n2 < 1 || num_slices < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad volume shape (%d, %d, %d) or slice count %d",
                n0, n1, n2, num_slices);
  if (out_mode != 1 && out_mode != 2)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "out_mode must be 1 or 2 (got %d)", out_mode);
  cudaError_t e = launch_volume_expand(sliced, sliced_old, num_slices, n0, (size_t)n1 * n2, out,
                                       out_mode, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "volume expansion kernel");
  return PTYCHO_OK;
}

int ptycho_volume_add_scaled(float* volume, const float* addend, int64_t count, int32_t divisor,
                             void* stream) {
  if (!volume || !addend)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "volume and addend must be non-null");
  if (count < 0 || divisor < 1)
    return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad count %lld or divisor %d", (long long)count,
                divisor);
  if (count == 0) return PTYCHO_OK;
  cudaError_t e = launch_volume_add_scaled(volume, addend, (size_t)count, divisor,
                                           static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "volume add kernel");
  return PTYCHO_OK;
}

int ptycho_volume_constraints(float* volume, int64_t count, float shrinkage,
                              int32_t apply_shrinkage, int32_t positivity, void* stream) {
  if (!volume) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "volume is null");
  if (count < 0) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "bad count %lld", (long long)count);
  if (count == 0 || (!apply_shrinkage && !positivity)) return PTYCHO_OK;
  cudaError_t e = launch_volume_constraints(volume, (size_t)count, shrinkage,
                                            apply_shrinkage ? 1 : 0, positivity ? 1 : 0,
                                            static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "volume constraint kernel");
  return PTYCHO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Gradient-descent batch for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc at all: an acquisition
// loop that fixes its device-memory budget when the microscope session starts
// and must not allocate (or block on an allocation) while patterns stream in,
// or a host application whose own allocator owns the GPU, so that memory taken
// behind its back would break its accounting. They cannot provide the
// workspace ptycho_gd_batch() needs. ptycho_gd_batch_noalloc() runs the same
// kernels with their scratch in the fixed-size array below instead, so the call
// itself allocates nothing.
//
//  - The array is kNoallocScratchBytes (32 MiB) of device memory that every GPU
//    holds from the moment it loads this library until the process exits.
//  - Its device address is looked up once per device (cudaGetSymbolAddress,
//    on the first call made with that device current); make that first call
//    before any stream capture.
//  - Every call on a device uses the same array. Two calls that may run at the
//    same time on the GPU (different streams or host threads) overwrite each
//    other's scratch: issue them in order on one stream.
//  - Within one call the kernels write every scratch byte before they read it,
//    so no part of the array has to start at zero and nothing is cleared
//    between calls. That holds only while no call reads what an earlier call
//    left behind, so the batch-chaining flags are refused here:
//    PTYCHO_FLAG_SPECTRUM_READY (would read a probe spectrum left by the
//    previous call, which may belong to another probe or geometry),
//    PTYCHO_FLAG_PREPARE_SPECTRUM (prepares one for such a read) and
//    PTYCHO_FLAG_KEEP_FARFIELD (keeps far fields for a position-correction call
//    that cannot be given this array).
namespace {
constexpr size_t kNoallocScratchBytes = size_t(32) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];
std::mutex g_noalloc_mu;
std::vector<void*> g_noalloc_addr;  // per device ordinal, nullptr until looked up
}  // namespace

extern "C" int ptycho_gd_batch_noalloc(const ptycho_geometry* g, void* object, void* probe,
                                       const float* amplitudes, const int32_t* amplitude_rows,
                                       const float* positions_px, const int32_t* position_rows,
                                       int32_t batch, float step_size, float normalization_min,
                                       int32_t fix_probe, const float* detector_mask,
                                       const void* propagators, float* error_accum,
                                       void* stream) {
  int st = check_geometry(g);
  if (st != PTYCHO_OK) return st;
  if (g->flags & (PTYCHO_FLAG_SPECTRUM_READY | PTYCHO_FLAG_PREPARE_SPECTRUM |
                  PTYCHO_FLAG_KEEP_FARFIELD))
    return fail(PTYCHO_ERR_INVALID_ARGUMENT,
                "ptycho_gd_batch_noalloc does not take PTYCHO_FLAG_SPECTRUM_READY, "
                "PTYCHO_FLAG_PREPARE_SPECTRUM or PTYCHO_FLAG_KEEP_FARFIELD (they pass data "
                "between calls through the scratch, which every call shares)");
  if (batch < 1) return fail(PTYCHO_ERR_INVALID_ARGUMENT, "batch must be >= 1 (got %d)", batch);
  const size_t need = ptycho_workspace_bytes(g, batch);
  if (need > kNoallocScratchBytes)
    return fail(PTYCHO_ERR_WORKSPACE,
                "batch of %d positions needs %zu bytes of scratch; the fixed no-allocation "
                "scratch holds %zu bytes (use fewer positions per call or ptycho_gd_batch "
                "with a workspace)",
                batch, need, kNoallocScratchBytes);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if ((size_t)dev >= g_noalloc_addr.size()) g_noalloc_addr.resize(dev + 1, nullptr);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
      g_noalloc_addr[dev] = p;
    }
    scratch = g_noalloc_addr[dev];
  }
  return ptycho_gd_batch(g, object, probe, amplitudes, amplitude_rows, positions_px,
                         position_rows, batch, step_size, normalization_min, fix_probe,
                         detector_mask, propagators, error_accum, scratch,
                         kNoallocScratchBytes, stream);
}
