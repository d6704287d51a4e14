/*
 * oopao_gb300 — C ABI of the GB300 (sm_103a) modulated pyramid wavefront
 * sensor and deformable-mirror influence-function projection.
 *
 * All array arguments are plain pointers.  "host" pointers are read during
 * the call only; "device" pointers must be CUDA device memory on the current
 * device.  `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  Every function returns OOPAO_OK (0) or an OOPAO_ERR_* code; the
 * message of the last failure on the calling thread is in oopao_last_error().
 * Compute calls are asynchronous with respect to the host.
 *
 * Layouts: 2-D maps are row-major [row][col]; complex values are interleaved
 * (re, im) float pairs; batched maps are [batch][row][col].
 *
 * Each entry point names the reference (cheritier/OOPAO) interface whose
 * computation it replaces; paths are relative to the OOPAO project root.
 */
#ifndef OOPAO_GB300_H
#define OOPAO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OOPAO_OK = 0,
  OOPAO_ERR_INVALID = 1,      /* bad argument (size, pointer, mode) */
  OOPAO_ERR_UNSUPPORTED = 2,  /* e.g. FFT size with a prime factor > 13 */
  OOPAO_ERR_CUDA = 3,         /* a CUDA runtime call failed */
  OOPAO_ERR_WORKSPACE = 4     /* workspace smaller than one batch item needs */
};

/* Library ABI version (incremented on any signature change). */
int oopao_abi_version(void);
/* Message of the last error on this thread ("" if none). */
const char* oopao_last_error(void);
/* Number of CUDA kernels this library has launched in the process
 * (instrumentation, no reference counterpart). */
unsigned long long oopao_launch_count(void);

/* ------------------------------------------------------------------------
 * Pyramid wavefront sensor plan.
 * Replaces the geometry built by Pyramid.__init__ (OOPAO/Pyramid.py:26-366):
 * FFT grid n_fft (:276-279), camera size cam (:285), centring phasor
 * (:342-344), complex64 mask (:368-391) and the modulation path (:1112-1139).
 * ------------------------------------------------------------------------ */
typedef struct oopao_pwfs_plan oopao_pwfs_plan;

/* mask_host: [n_fft*n_fft] complex64 (interleaved floats), the pyramid mask
 *   (already multiplied by any spatial filter).
 * tt_path_host: [2*n_theta] modulation points (x_k, y_k) in lambda/D, or NULL
 *   with n_theta == 1 for the non-modulated sensor.
 * tt_scale: telescope.resolution / telescope.initial_resolution (:336-339).
 * psf_centering: 1 = mask centred on 4 pixels (phasor), 0 = on 1 pixel
 *   (fftshift of the focal field, :632-639). */
int oopao_pwfs_plan_create(oopao_pwfs_plan** plan, int res, int n_fft, int cam, int n_theta,
                           const float* mask_host, const double* tt_path_host, double tt_scale,
                           int psf_centering);
int oopao_pwfs_plan_destroy(oopao_pwfs_plan* plan);

/* Pupil amplitude sqrt(src.intensity / nTheta) [res*res] (OOPAO/Pyramid.py:674). */
int oopao_pwfs_set_amplitude(oopao_pwfs_plan* plan, const float* amp_host);
/* Several Fourier masks measured together (the Bi-O Edge sensor's four,
 * OOPAO/BioEdge.py:510-544): masks_host = [n_masks][n_fft][n_fft] complex64
 * (1 to 8; mask 0 replaces the plan's mask).  The forward transforms of each
 * modulation point are computed once; measure then writes frame
 * [batch][n_masks][cam][cam] and raw [batch][n_masks][n_fft][n_fft].  With
 * n_masks > 1 the plan needs a compile-time variant with one stage-B
 * butterfly per thread (else OOPAO_ERR_UNSUPPORTED at measure) and the
 * tangent/adjoint entry points return OOPAO_ERR_UNSUPPORTED. */
int oopao_pwfs_set_masks(oopao_pwfs_plan* plan, int n_masks, const float* masks_host);
int oopao_pwfs_n_masks(const oopao_pwfs_plan* plan);
/* Optional per-point weights [n_theta] (Pyramid.weight_vector, :750-755);
 * NULL restores the plain sum.  The device copy stays allocated until the
 * plan is destroyed, so a captured graph may keep its address; switching
 * the weights off or on does not free or move it. */
int oopao_pwfs_set_weights(oopao_pwfs_plan* plan, const float* weights_host);
/* Launch shape (autotuner hook, no reference counterpart): lines per CTA of
 * the generic FFT passes (0 keeps a value) and the number of partial sums
 * over modulation points (must divide n_theta; 0 = automatic, -1 keeps). */
int oopao_pwfs_set_launch(oopao_pwfs_plan* plan, int rows_per_cta, int cols_per_cta,
                          int inv_rows_per_cta, int ksplit);
/* Bytes of row/column FFT intermediates one pass may hold (no reference
 * counterpart).  oopao_pwfs_measure cuts a batch into passes of whole items
 * (or whole groups of modulation points) of at most this size; a budget
 * under the L2 size keeps them L2-resident between the three FFT passes.
 * 0 restores the default (4 GiB). */
int oopao_pwfs_set_pass_budget(oopao_pwfs_plan* plan, size_t bytes);

/* Kernel variant (autotuner hook, no reference counterpart): 0 = generic
 * runtime-planned kernels (any n_fft whose prime factors are <= 13),
 * 1..oopao_pwfs_num_variants = compile-time two-stage FFT plans for this
 * n_fft (a new plan starts on the fastest one measured for its n_fft;
 * oopao_pwfs_get_variant reports it).  An index beyond the count
 * returns OOPAO_ERR_UNSUPPORTED.  variant_info fills info[6] with
 * (R1, R2, threads per line, row / column / row-inverse lines per CTA). */
int oopao_pwfs_set_variant(oopao_pwfs_plan* plan, int variant);
/* Device status word of the plan's kernels, read synchronously and reset:
 * 0, or the code of a bounded wait that timed out (the kernel then stopped
 * without finishing its work; the results of that call are invalid). */
int oopao_pwfs_device_status(oopao_pwfs_plan* plan, int* code);
int oopao_pwfs_get_variant(const oopao_pwfs_plan* plan);
int oopao_pwfs_num_variants(const oopao_pwfs_plan* plan);
int oopao_pwfs_variant_info(const oopao_pwfs_plan* plan, int variant, int* info);

/* Two-pass propagation for masks that factorise per axis.  The reference's
 * single path (pyramid_transform, OOPAO/Pyramid.py:612-646) applies the
 * N x N mask between full 2-D transforms; when the plan's mask equals
 * mcol[r] * mrow[c] within float32 rounding (the four-face mask with one
 * shift for all faces, no rooftop, no rotation: OOPAO/Pyramid.py:453-480)
 * the filter splits into a row filter shared by the points with equal x_k
 * and a column filter per point, and oopao_pwfs_measure / oopao_pwfs_jvp run
 * two passes instead of three.  Same results within float32 round-off.
 * set_separable(plan, 0) forces the three-pass path; set_separable(plan, i)
 * with 1 <= i <= num_separable selects compile-time two-pass plan i (radix
 * order, columns per CTA) and uses the two passes whenever they apply (a new
 * plan starts on plan 1).  separable() returns 1 when a measure call without
 * a focal-plane frame takes the two-pass path, 2 when every mask of the plan
 * varies along one focal-plane axis only (the Bi-O Edge knife edges without
 * tip/tilt shifts, OOPAO/BioEdge.py:331-392) and a call takes the one-axis
 * path (filtered lines of that axis only, no column transform), else 0;
 * set_separable(plan, 0) turns both off. */
int oopao_pwfs_set_separable(oopao_pwfs_plan* plan, int enable);
int oopao_pwfs_separable(const oopao_pwfs_plan* plan);
int oopao_pwfs_num_separable(const oopao_pwfs_plan* plan);
/* How a measure call of `batch` items without raw data or focal frame is
 * launched (instrumentation, no reference counterpart): info[4] = (1 if the
 * two-pass path runs, row-transform groups, partial slots over modulation
 * points, items per chunk). */
int oopao_pwfs_pass_info(const oopao_pwfs_plan* plan, int batch, int* info);

/* Bytes of device workspace oopao_pwfs_measure needs for `batch` items
 * processed in one chunk (a smaller workspace makes it loop over chunks;
 * it must hold at least one item). */
size_t oopao_pwfs_workspace_bytes(const oopao_pwfs_plan* plan, int batch);

/* Modulated propagation + detector binning.
 * Replaces Pyramid.wfs_measure / pyramid_transform (OOPAO/Pyramid.py:612-833)
 * and the noise-free camera sum-binning (Pyramid.__mul__ :1178-1203,
 * tools.set_binning OOPAO/tools/tools.py:464-483).
 * opd: device [batch][res][res] float32; the phase is opd*phase_scale
 *   (phase_scale = 2*pi/lambda for an OPD in metres, 1 for a phase in rad).
 * frame: device [batch][cam][cam] float32 (required).
 * raw: device [batch][n_fft][n_fft] float32 raw_data, or NULL. */
int oopao_pwfs_measure(const oopao_pwfs_plan* plan, const float* opd, double phase_scale,
                       int batch, float* frame, float* raw, void* workspace,
                       size_t workspace_bytes, void* stream);

/* oopao_pwfs_measure plus the focal-plane (modulation) camera image.
 * Replaces the modulation_camera_em list of pyramid_transform
 * (OOPAO/Pyramid.py:642: the focal field F/N of every modulation point) and
 * its use by a focal-plane camera (Pyramid.__mul__ :1182-1190:
 * sum over points of |F/N|^2).
 * focal: device [batch][n_fft][n_fft] float32, overwritten; F is the focal
 * field before the pyramid mask (after the 1-pixel-centring shift when
 * psfCentering is off).  Summed with float atomics, so the last bits of
 * focal depend on the order of the additions; frame and raw do not. */
int oopao_pwfs_measure_focal(const oopao_pwfs_plan* plan, const float* opd, double phase_scale,
                             int batch, float* frame, float* raw, float* focal, void* workspace,
                             size_t workspace_bytes, void* stream);

/* Allocation-free variant of oopao_pwfs_measure.  It has no counterpart in
 * the reference.  It is for callers that cannot allocate device memory while
 * they measure: a real-time control loop that forbids allocation once it
 * runs, or a host framework that owns the GPU allocator.  The FFT
 * intermediates live in a 64 MiB array compiled into the library, which every
 * GPU that loads the library holds until the process exits; nothing is
 * allocated or freed by this call.  Arguments as oopao_pwfs_measure, without
 * the workspace.
 * - A plan whose smallest pass (one group of modulation points of one item)
 *   needs more than 64 MiB is rejected with OOPAO_ERR_WORKSPACE.
 * - The first call on a device looks up the array's device address (set-up,
 *   once per device, with that device current); make that first call before
 *   any stream capture.
 * - All calls share the one array: calls whose kernels overlap on the GPU
 *   (other streams, other host threads) race.  Serialise them.
 * - The plan itself is created (and allocated) beforehand at set-up time;
 *   per-kernel profiling must be off. */
int oopao_pwfs_measure_noalloc(const oopao_pwfs_plan* plan, const float* opd, double phase_scale,
                               int batch, float* frame, float* raw, void* stream);

/* Per-kernel timing (instrumentation, no reference counterpart): when
 * enabled, every oopao_pwfs_measure records CUDA events around its four
 * kernels (row FFT, column FFT/mask/IFFT, row IFFT/|.|^2, binning) on its
 * stream.  profile_read waits for the last event, returns the summed
 * milliseconds and launch counts per kernel ([4] each) and clears them. */
int oopao_pwfs_set_profiling(oopao_pwfs_plan* plan, int enable);
int oopao_pwfs_profile_read(oopao_pwfs_plan* plan, double* ms, int* launches);

/* Signal-processing setup (Pyramid.initialization / signalProcessing,
 * OOPAO/Pyramid.py:541-589, :835-926, grabQuadrant :946-961).
 * mode: 0 slopesMaps, 1 slopesMaps_incidence_flux, 2 slopesMaps_camera_flux,
 *       3 fullFrame, 4 fullFrame_incidence_flux, 5 fullFrame_camera_flux,
 *       6 fullFrame_sum_flux.
 * n_quad: quadrant size (slopes modes); quad_origin_host: [8] (row, col) of
 *   the top-left pixel of quadrants 1..4 in the camera frame.
 * valid_host: [n_quad*n_quad] validI4Q (slopes) or [cam*cam] validSignal
 *   (full frame), 0/1 bytes.
 * ref2d_host: referenceSignal_2D [2*n_quad*n_quad] or [cam*cam], or NULL (0).
 * norma_const: the flux normalisation of the *_incidence_flux modes. */
int oopao_pwfs_set_signal_processing(oopao_pwfs_plan* plan, int mode, int n_quad,
                                     const int* quad_origin_host, const unsigned char* valid_host,
                                     const float* ref2d_host, double slopes_units,
                                     double norma_const);
/* Number of entries of wfs.signal for the current valid map. */
int oopao_pwfs_n_signal(const oopao_pwfs_plan* plan);

/* wfs.signal_2D / wfs.signal from camera frames (signalProcessing).
 * frame: device [batch][cam][cam]; signal_2d: device [batch][2*n_quad][n_quad]
 * (slopes) or [batch][cam][cam] (full frame); signal: device
 * [batch][n_signal]; norma: device [batch] or NULL. */
int oopao_pwfs_signal(const oopao_pwfs_plan* plan, const float* frame, int batch,
                      float* signal_2d, float* signal, float* norma, void* stream);

/* ------------------------------------------------------------------------
 * Deformable mirror influence-function projection.
 * Replaces the dm.coefs setter OPD = modes @ coefs
 * (OOPAO/DeformableMirror.py:651-686).
 * modes_t: device [n_act][n_pix] float32 (the transpose of dm.modes).
 * coefs: device [n_act][batch] float32 (the layout of a 2-D dm.coefs).
 * opd: device [batch][n_pix] float32 = (modes @ coefs)^T * scale.
 * ------------------------------------------------------------------------ */
int oopao_dm_opd_f32(const float* modes_t, const float* coefs, int n_act, int n_pix, int batch,
                     float scale, float* opd, void* stream);
/* BF16 tensor-core projection (tcgen05 MMA, TMA-fed tiles, FP32
 * accumulation), same result layout as oopao_dm_opd_f32 (plus an optional
 * base).  modes: device [n_pix][n_act_pad] BF16 (K-major, zero padded,
 * n_act_pad a multiple of 64), built once by oopao_dm_modes_bf16 from the
 * FP32 modes_t.  The coefficients enter as two BF16 terms (hi = bf16(c),
 * lo = bf16(c - hi)) summed in the FP32 accumulator, so only the IF matrix
 * is rounded to BF16.  Batches of 1 to 4 (a closed-loop step) use a
 * streaming GEMV over the BF16 rows with FP32 coefficients instead of the
 * tensor cores.  workspace: device, 256-byte aligned,
 * oopao_dm_bf16_workspace_bytes(n_act_pad, batch) bytes; its first int
 * holds 0 after the call, or the code of a pipeline wait that timed out. */
int oopao_dm_modes_bf16(const float* modes_t, int n_act, int n_pix, int n_act_pad, void* modes_out, void* stream);
size_t oopao_dm_bf16_workspace_bytes(int n_act_pad, int batch);
int oopao_dm_opd_bf16(const void* modes, int n_act_pad, const float* coefs, int n_act, int n_pix, int batch,
                      float scale, const float* base, float* opd, void* workspace, size_t workspace_bytes,
                      void* stream);
/* The same with the GEMM's batch tile chosen by the caller (autotuner hook,
 * no reference counterpart): tile_n = 64 or 128 columns per CTA tile, or 0
 * for the automatic rule (GEMV up to 4 columns, 64 up to 64, else 128); a
 * non-zero tile_n uses the tensor cores at every batch. */
int oopao_dm_opd_bf16_tiled(const void* modes, int n_act_pad, const float* coefs, int n_act, int n_pix, int batch,
                            float scale, const float* base, float* opd, void* workspace, size_t workspace_bytes,
                            int tile_n, void* stream);
/* The projection at FP32 accuracy on the tensor cores (tcgen05
 * kind::tf32), for IFs that neither factorise nor are stored in BF16.
 * oopao_dm_modes_tf32x2: modes_t [n_act][n_pix] f32 -> out device f32
 * [2][n_pix][n_act_pad] (n_act_pad a multiple of 32): the IFs rounded to TF32,
 * then the FP32 remainders.  oopao_dm_opd_tf32x3: opd = (modes @ coefs)^T *
 * scale (+ base) from three TF32 products (hi*hi + hi*lo + lo*hi, FP32
 * accumulation), relative error ~1e-6 against float64; same layouts and
 * workspace rules as oopao_dm_opd_bf16 (the error word at its head). */
int oopao_dm_modes_tf32x2(const float* modes_t, int n_act, int n_pix, int n_act_pad, float* out, void* stream);
size_t oopao_dm_tf32_workspace_bytes(int n_act_pad, int batch);
int oopao_dm_opd_tf32x3(const float* modes2, int n_act_pad, const float* coefs, int n_act, int n_pix, int batch,
                        float scale, const float* base, float* opd, void* workspace, size_t workspace_bytes,
                        void* stream);

/* Separable influence functions (DeformableMirror.modesComputation,
 * OOPAO/DeformableMirror.py:572-600, with anamorphosisAngle = 0 on a
 * Cartesian actuator grid): modes[y*res + x][a] = gx[i_a][x] * gy[j_a][y].
 * opd[b][y][x] = scale * sum_j gy[j][y] sum_i C_b[j][i] gx[i][x] + base,
 * C_b[j][i] = coefs[grid_act[j*nx + i]][b] (grid_act < 0: no actuator).
 * gx device [nx][res], gy [ny][res], grid_act [ny*nx] int32, coefs
 * [n_act][batch]; same output layout as oopao_dm_opd_f32.  ws: at least
 * oopao_dm_sep_workspace_bytes(ny, res, batch) bytes.  One launch when
 * nx*ny + 16*nx + 80*ny <= 24576 (the coefficient grid and one block of the
 * factors fit in shared memory), two otherwise. */
size_t oopao_dm_sep_workspace_bytes(int ny, int res, int batch);
int oopao_dm_opd_sep_f32(const float* gx, const float* gy, const int* grid_act, int nx, int ny, const float* coefs,
                         int n_act, int res, int batch, float scale, const float* base, float* opd, void* ws,
                         size_t ws_bytes, void* stream);

/* opd = (modes @ coefs)^T * scale + base: the DM shape added to an incoming
 * OPD in one pass (DeformableMirror.relay, OOPAO/DeformableMirror.py:441-447:
 * src.OPD_no_pupil += dm.OPD).  base: device [batch][n_pix] or NULL. */
int oopao_dm_opd_acc_f32(const float* modes_t, const float* coefs, int n_act, int n_pix, int batch,
                         float scale, const float* base, float* opd, void* stream);

/* ------------------------------------------------------------------------
 * Closed-loop step (tutorials/AO_closed_loop_Pyramid_WFS.py:601-639,
 * OOPAO/closed_loop/run_cl.py:176-217).  `step` is a device int counter:
 * oopao_cl_screen reads it, oopao_cl_integrate advances it, so a captured
 * CUDA graph of one step replays later steps without host updates.
 * ------------------------------------------------------------------------ */
/* Frozen-flow turbulence: opd[res][res] = sum over layers of the periodic
 * screen q (device [heights[q]][widths[q]], OPD in m) sampled bilinearly at
 * (y0[q] + i + vy[q]*step, x0[q] + j + vx[q]*step) (pixels).  Host arrays of
 * n_layers <= 35 entries. */
int oopao_cl_screen(int n_layers, const float* const* screens, const int* heights, const int* widths,
                    const float* y0, const float* x0, const float* vy, const float* vx, int res,
                    const int* step, float* opd, void* stream);
/* Integrator: coefs -= gain * R @ s (R device [n_act][n_sig]); advances
 * *step by one when step is not NULL. */
int oopao_cl_integrate(const float* R, const float* s, int n_act, int n_sig, float gain, float* coefs,
                       int* step, void* stream);
/* Modal commands with optical-gain compensation (the reference's GSC
 * tutorial, M2C @ diag(1/og) @ M @ s): y[m] = (M @ s)[m] / og[m] once
 * *step >= og_start, (M @ s)[m] before or when og is NULL.  M device
 * [n_modes][n_sig] float32, og device float64 [n_modes] (the gains of
 * oopao_gsc_optical_gains), y device [n_modes]; step may be NULL (always
 * compensated). */
int oopao_cl_modal(const float* M, const float* s, int n_modes, int n_sig, const double* og, int og_start,
                   const int* step, float* y, void* stream);
/* Residual wavefront RMS over pupil pixels idx[npup] (device) written to
 * out[*step] (device, out_len entries). */
int oopao_cl_pupil_rms(const float* opd, const int* idx, int npup, const int* step, float* out, int out_len,
                       void* stream);

/* One update of the infinite-phase-screen atmosphere and its OPD for an
 * on-axis source.  Replaces Atmosphere.update -> updateLayer / add_row
 * (OOPAO/Atmosphere.py:410-531) and fill_OPD_support (:589-622).
 * maps: device float64 [2][n_layers][n][n] ping-pong phase maps (radians,
 *   n = res + 6); the current maps are in the first half on entry and exit.
 * sched: device [n_steps][n_layers][slots] entries {active, dx, dy,
 *   normal row} of int32: the one-pixel moves (add_row) of each step, at most
 *   `slots` (even) per step; buff: device float64 [n_steps][n_layers][2]
 *   sub-pixel offsets (x, y) after each step, or NULL for the unshifted maps.
 * A [n_outer][n_inner], B [n_outer][n_outer]: float64 extrusion matrices;
 *   inner_idx / outer_idx: map indices of the Z and X rings; normals:
 *   float64 [rows][n_outer] drawn by the host.
 * mirror: device float32 [n_layers][n][n] scratch, the maps rounded to
 *   float32 for the interpolation;
 * range: device float64 [n_layers][32][2] scratch (partial value ranges of
 *   each map); at most 64 layers;
 * scale: device float64 [n_layers] = lambda/2pi * sqrt(fractional r0);
 * opd: device float32 [res][res] output; step: device int32, the step whose
 *   entries are used, incremented at the end when `advance`; err: device
 *   int32 set to 1 when *step is outside [0, n_steps) (nothing moves then). */
int oopao_atm_update(double* maps, float* mirror, int n_layers, int n, int slots, const void* sched,
                     const double* buff, int n_steps, const double* A, const double* B, const int* inner_idx, const int* outer_idx,
                     int n_inner, int n_outer, const double* normals, double* range, const double* scale, int res,
                     float* opd, int* step, int advance, int* err, void* stream);

/* Boiling of the layers (AR(1) decorrelation; replaces Atmosphere.apply_boiling,
 * OOPAO/Atmosphere.py:387-408, called by updateLayer :457 before the frozen-flow
 * moves): maps[layers[k]] = alpha[k] * maps[layers[k]] + beta[k] * phi[t][k]
 * for k < n_boil, in float64 with separately rounded products.  Run it before
 * oopao_atm_update of the same step, on the same stream.
 * maps: device float64 [n_layers][n][n] (the first ping-pong half);
 * phi: device float64 [n_steps][n_boil][n][n] new screens;
 * layers, alpha, beta: HOST arrays [n_boil] (layers increasing);
 * step: device int32 counter selecting t (as oopao_atm_update: err set to 1
 *   and nothing changes outside [0, n_steps)), or NULL with n_steps = 1. */
int oopao_atm_boil(double* maps, int n_layers, int n, const double* phi, int n_boil, const int* layers,
                   const double* alpha, const double* beta, const int* step, int n_steps, int* err, void* stream);

/* Adjoint of the projection (no reference counterpart; used by the
 * gradients of wfs.signal with respect to dm.coefs):
 * out[a][b] = scale * sum_p modes_t[a][p] * g[b][p];
 * g: device [batch][n_pix]; out: device [n_act][batch]. */
int oopao_dm_vjp_f32(const float* modes_t, const float* g, int n_act, int n_pix, int batch, float scale,
                     float* out, void* stream);

/* ------------------------------------------------------------------------
 * Tangent (JVP) and adjoint (VJP) of the propagation.  No reference
 * counterpart: the reference obtains derivatives only by finite push-pull
 * differences (OOPAO/calibration/InteractionMatrix.py:117-158).  Available
 * for n_fft in {72, 112, 128, 264, 504, 1920} (compile-time plans) on plans
 * with one mask, otherwise OOPAO_ERR_UNSUPPORTED.  Workspace: oopao_pwfs_ad_workspace_bytes.
 * ------------------------------------------------------------------------ */
size_t oopao_pwfs_ad_workspace_bytes(const oopao_pwfs_plan* plan, int batch);
/* dframe[b] = d frame / d opd at opd0 applied to dopd[b].
 * opd0: device [opd0_batch][res][res] operating points (opd0_batch 1 = one
 * point shared by all tangents, e.g. an interaction matrix at a flat
 * wavefront; or batch); dopd: device [batch][res][res]; dframe: device
 * [batch][cam][cam].  The phase is opd*phase_scale. */
int oopao_pwfs_jvp(const oopao_pwfs_plan* plan, const float* opd0, int opd0_batch, const float* dopd,
                   double phase_scale, int batch, float* dframe, void* workspace, size_t workspace_bytes,
                   void* stream);
/* opd_bar[b] = (d frame / d opd at opd[b])^T fbar[b]; opd, opd_bar: device
 * [batch][res][res]; fbar: device [batch][cam][cam].  Each modulation
 * point's field is recomputed, not stored. */
int oopao_pwfs_vjp(const oopao_pwfs_plan* plan, const float* opd, const float* fbar, double phase_scale,
                   int batch, float* opd_bar, void* workspace, size_t workspace_bytes, void* stream);
/* Tangent and adjoint of signalProcessing for slopesMaps and
 * slopesMaps_incidence_flux (quotient rule through the normalisation).
 * frame0: device [frame0_batch][cam][cam] operating-point frames. */
int oopao_pwfs_signal_jvp(const oopao_pwfs_plan* plan, const float* frame0, int frame0_batch,
                          const float* dframe, int batch, float* dsignal_2d, float* dsignal, void* stream);
int oopao_pwfs_signal_vjp(const oopao_pwfs_plan* plan, const float* frame0, int frame0_batch,
                          const float* sbar, int batch, float* fbar, void* stream);

/* ------------------------------------------------------------------------
 * Gain-sensing camera: optical gains of the modulated pyramid from its
 * full-resolution focal-plane frame (OOPAO/GainSensingCamera.py:13-199,
 * Chambouleyron et al. 2021).  The plan holds the mask, its centred
 * spectrum, the basis product (float32 [n_modes][n][n], the reference's
 * split_basis_product :158-173 for a real basis) and the calibration.
 * Sizes: n = mask size (even, prime factors <= 13).
 * ------------------------------------------------------------------------ */
typedef struct oopao_gsc_plan oopao_gsc_plan;
enum { OOPAO_GSC_IR_CALIB = 0, OOPAO_GSC_SENSI_CALIB = 1, OOPAO_GSC_BASIS_PRODUCT = 2, OOPAO_GSC_MODE_POWER = 3 };
/* GainSensingCamera.__init__ (:15-76).  mask_host: complex64 [n][n]
 * (interleaved re, im), the pyramid's wfs.mask. */
int oopao_gsc_plan_create(oopao_gsc_plan** plan, int n, int n_modes, const float* mask_host);
int oopao_gsc_plan_destroy(oopao_gsc_plan* plan);
/* Workspace of calibrate (batch 1) and optical_gains (batch frames). */
size_t oopao_gsc_workspace_bytes(const oopao_gsc_plan* plan, int batch);
/* Basis product of split_basis_product (:158-173) and padder (:140-147):
 * basis: device float32 [n_modes][n0][n0] (the reference's [n0, n0, modes]
 * transposed), zero-padded by (n - n0)/2 on each side.  Rows are stored
 * divided by the mode's power (the gains do not depend on it).  Any
 * workspace of at least n*n*8 bytes; larger ones transform more modes per
 * launch. */
int oopao_gsc_set_basis(oopao_gsc_plan* plan, const float* basis, int n0, void* workspace, size_t workspace_bytes,
                        void* stream);
/* calibration (:78-95): frame = device float32 [n][n] focal-plane frame at
 * the working point (normalised to unit sum inside).  Stores IR_calib,
 * ifft3(IR_calib) and sensi_calib in the plan. */
int oopao_gsc_calibrate(oopao_gsc_plan* plan, const float* frame, void* workspace, size_t workspace_bytes,
                        void* stream);
/* compute_optical_gains (:104-120) for `batch` frames: frames device float32
 * [batch][n][n]; og device float64 [batch][n_modes]; optional sensitivity
 * device complex128 [batch][n_modes] (sensitivity(IR_sky, IR_calib)) and ir
 * device float32 [batch][n][n] (IR_sky).  Status OOPAO_ERR_INVALID before
 * a calibration. */
int oopao_gsc_optical_gains(const oopao_gsc_plan* plan, const float* frames, int batch, double* og,
                            double* sensitivity, float* ir, void* workspace, size_t workspace_bytes, void* stream);
/* Device-to-device copy of a plan array: OOPAO_GSC_IR_CALIB float32 [n][n],
 * OOPAO_GSC_SENSI_CALIB complex128 [n_modes], OOPAO_GSC_BASIS_PRODUCT
 * float32 [n_modes][n][n] with each row divided by the mode's power,
 * OOPAO_GSC_MODE_POWER float64 [n_modes] (sum of the mode's squares, which
 * is also the row sum of its basis product). */
int oopao_gsc_read(const oopao_gsc_plan* plan, int what, void* dst, void* stream);

/* ------------------------------------------------------------------------
 * Detector readout, the stages without random draws (the noise draws are
 * made by the caller between the calls).  frames: device float32
 * [nframes][npix], rewritten in place; one frame per CTA.
 * ------------------------------------------------------------------------ */
/* Detector.set_saturation (OOPAO/Detector.py:219-224): max_out device
 * float32 [nframes] receives each frame's maximum before the clip to
 * [0, fwc] (the saturation percentage and warning are the caller's). */
int oopao_det_saturate(float* frames, int nframes, int npix, float fwc, float* max_out, void* stream);
/* The end of Detector.readout (OOPAO/Detector.py:304-318), in its order:
 * frame *= gain (pass 1 for an EMCCD, whose gain acts earlier); if bits > 0
 * the ADC of digitalization (:226-238): fwc <= 0 scales by 2^bits over the
 * frame maximum, else frame / fwc * (2^bits - 1) clipped to
 * [clip_zero ? 0 : -inf, 2^bits - 1]; log10 if log_scale; the cast to the
 * output precision of set_output_precision (:192-213), out_bits 8/16/32/64
 * for the unsigned types (truncation toward zero, values outside the type
 * wrap modulo 2^out_bits) or 0 for floating point; minus bg_map (device
 * float32 [npix] or NULL, remove_bakground :266-271).  max_out (device
 * float32 [nframes] or NULL) receives each frame's maximum after the gain,
 * for the ADC saturation warning. */
int oopao_det_readout_tail(float* frames, int nframes, int npix, float gain, int bits, float fwc, int clip_zero,
                           int log_scale, int out_bits, const float* bg_map, float* max_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* OOPAO_GB300_H */
