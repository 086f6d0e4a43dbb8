/*
 * wavebit_gb300 — C ABI of libwbgpu.so, the GB300 (sm_103a) RCWA raster layer path.
 *
 * The reference (fieldalgo/wavebit, pure Python) has no native interface; these entry points
 * are what its RCWA backend seam would bind through ctypes. Each declaration names the
 * reference function whose role it takes (paths inside src/wavebit).
 *
 * Conventions
 *   - Every function returns WB_OK (0) or a WB_E_* code; wb_last_error() gives the message
 *     of the calling thread's last failure.
 *   - Complex numbers are interleaved (re, im) doubles (wb_complex).
 *   - Matrices are column-major: element (i, j) of an N x N matrix is at [i + j * N].
 *   - Rasters are row-major (L, ny, nx): element (layer, y, x) at [(layer * ny + y) * nx + x],
 *     rows along the second lattice axis (v), columns along the first (u).
 *   - Orders are flattened i = n * n_u + m (m along u fastest), N = (2hu+1)(2hv+1).
 *   - Layers are listed entry face first: index 0 is the layer that touches the superstrate.
 *   - Device entry points take caller-owned device pointers and a cudaStream_t (as void*);
 *     they are asynchronous on that stream. The library never frees caller memory; its own
 *     scratch comes from the handle's arena, sized at wb_create.
 *   - A handle is used by one host thread at a time.
 */
#ifndef WAVEBIT_GB300_H
#define WAVEBIT_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define WB_OK 0
#define WB_E_INVALID 1     /* bad argument (reference: ValidationError, code 'input.invalid') */
#define WB_E_NOMEM 2       /* the request does not fit the handle's HBM budget */
#define WB_E_SINGULAR 3    /* an exact zero pivot (reference: NumericalError 'rcwa.singular') */
#define WB_E_NOCONV 4      /* the eigenvalue iteration hit its cap (LAPACK zgeev info > 0) */
#define WB_E_NONFINITE 5   /* NaN/Inf in a result (reference: NumericalError 'rcwa.nonfinite') */
#define WB_E_CUDA 6        /* a CUDA runtime error */

/* per-solve status bits written on the device */
#define WB_ST_SINGULAR 1
#define WB_ST_NOCONV 2
#define WB_ST_NONFINITE 4
#define WB_ST_GRAZING 8    /* min|w| < 1e-9 max|w|: the reference rebuilds such a layer
                              (rcwa/_engine/solve_2d.py:2463-2482); the result is flagged */

#define WB_PRECISION_FP64 0        /* IEEE FP64 throughout */
#define WB_PRECISION_MIXED 1       /* FP32 eigen-solve brought to FP64 accuracy by Newton steps
                                      against the FP64 operator; FP32 cascade whose amplitudes are
                                      refined against the double-float interface equations */
#define WB_PRECISION_MIXED_FP32 2  /* double-float (2 x FP32) eigen-solve, unrefined FP32 cascade
                                      (~1e-5) */
#define WB_PRECISION_MIXED_DF64 3  /* double-float eigen-solve and cascade */
#define WB_PRECISION_MIXED_DF64_EIG 4  /* double-float eigen-solve, refined FP32 cascade */

typedef struct { double re, im; } wb_complex;
typedef struct wb_handle wb_handle;

/* Version of this ABI (major * 100 + minor): 2.0 = the precision codes above (WB_PRECISION_MIXED
 * is the FP32 eigen-solve with Newton steps), wb_smm_solve and wb_workspace_bytes; 2.1 adds
 * wb_assemble_li_integrated and wb_scattering_matrix; 2.2 adds the reverse passes wb_smm_solve_vjp,
 * wb_layer_modes_vjp and wb_assemble_li_vjp, the tunable WB_TUNE_HRD_BLOCKED, and wb_layer_modes
 * with WB_PRECISION_MIXED runs the FP32 eigen-solve refined by Newton steps (before 2.2: the
 * double-float one). */
int wb_version(void);

/* Message of the calling thread's last failure, NUL-terminated, truncated to len. */
int wb_last_error(char* buf, size_t len);

/* Create a handle on `device` whose scratch arena may use up to hbm_budget bytes
 * (0 = 80% of the free device memory). Replaces the per-run solver objects the reference
 * builds in rcwa/_adapt.py:432-490 (build_solver) and rcwa/_factory.py:6-64. */
int wb_create(int device, size_t hbm_budget, wb_handle** out);
int wb_destroy(wb_handle* h);

/* Grow the handle's scratch arena to at least `bytes` now (within its budget), so that no
 * later call on the handle allocates. Serving loops call it once per worker at start-up. */
int wb_reserve(wb_handle* h, size_t bytes);

/* Order windows: every entry point takes orders (hu, hv) with 0 <= hv <= 42 and
 * N = (2hu+1)(2hv+1) <= 3228 (the largest windows the kernels hold on chip) and refuses others
 * with WB_E_INVALID; wb_workspace_bytes returns 0 for them. */

/* Bit-exact harmonic tables: labels_u[2hu+1] = -hu..hu, labels_v likewise; toeplitz_u
 * [(2hu+1)^2] = r - c + 2hu row-major, toeplitz_v likewise. Host memory, no handle needed.
 * Reference: rcwa/_engine/engine.py:953-993 (_separable_kxy order labels),
 * rcwa/_engine/factorization.py:276-286 (_circulant_index), :358-366 (_toeplitz_positions). */
int wb_build_indices(int hu, int hv, int32_t* labels_u, int32_t* labels_v, int32_t* toeplitz_u,
                     int32_t* toeplitz_v);

/* Stage A: Li-rule (fixed nesting) convolution matrices of L rasters, sampled coefficients.
 * eps: device (L, ny, nx); epx, epy, epz_i: device (L, N, N) column-major; status: device
 * int32 (1) or NULL. Reference: rcwa/_engine/factorization.py:915-941
 * (to_conv_mat_raster_sampled) with :369-440, :504-671. */
int wb_assemble_li(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                   wb_complex* epx, wb_complex* epy, wb_complex* epz_i, int32_t* status, void* stream);

/* Stage A with integrated (closed-form segment) coefficients, Li fixed nesting. eps: device
 * (L, ny, nx) compressed cells, each pixel standing for one block of equal neighbours of the
 * raster; x_edges: device (L, nx) right edges of the column blocks on the unit cell, y_edges:
 * device (L, ny) those of the row blocks, increasing, the last one 1 (the record
 * compression_indices returns). Outputs as wb_assemble_li. Reference:
 * rcwa/_engine/factorization.py:3181-3206 (to_conv_mat_raster_integrated), :443-501
 * (_segment_bounds, _segment_series), :3005-3045 (compression_indices). */
int wb_assemble_li_integrated(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, const double* x_edges,
                              const double* y_edges, int hu, int hv, wb_complex* epx, wb_complex* epy,
                              wb_complex* epz_i, int32_t* status, void* stream);

/* Stage B: eigenmodes of n_pairs layers. conv: device (n_conv, 3, N, N) slots epx, epy, epz_i;
 * pair_layer: device (n_pairs) index into conv, each in [0, n_conv) (device data: the library
 * cannot read it before the kernels do, so the caller keeps it in range); kx, ky: device
 * (n_pairs, N) normalised order wavevectors. Outputs (device): w (n_pairs, 2N) eigenvalues of Omega^2, q (n_pairs, 2N),
 * W and V (n_pairs, 2N, 2N) column-major, status (n_pairs). precision: WB_PRECISION_FP64 for
 * the FP64 eigen-solve, WB_PRECISION_MIXED for the FP32 eigen-solve refined by Newton steps on
 * the FP64 operator (the mixed form's stage B; FP64-class eigenpairs), any other WB_PRECISION_*
 * for the double-float eigen-solve.
 * Reference: rcwa/_engine/solve_2d.py:2303-2460 (layer_modes_2d, no exceptional-point
 * rebuilds), _common/conventions.py:186-249 (mode_q), _common/backend.py:1767-1812 (eig). */
int wb_layer_modes(wb_handle* h, int n_pairs, int hu, int hv, const wb_complex* conv,
                   const int32_t* pair_layer, const double* kx, const double* ky, wb_complex* w,
                   wb_complex* q, wb_complex* W, wb_complex* V, int32_t* status, int precision,
                   void* stream);

/* One batch of whole solves (stages B and C). Every array is a device pointer.
 *   conv        (n_conv, 3, N, N) from wb_assemble_li, any layers of any stacks
 *   layer_index (B, L) into conv, entry face first, each in [0, n_conv) (not checked on the
 *               device: the caller keeps it in range);  thickness (B, L), in wavelength units
 *   wavelength (B); period (B, 2); theta, phi (B) radians (real; lossless superstrate)
 *   eps_top, eps_bot (B); pol (B, 2) = (a_s, a_p), unit norm
 * Outputs: R, T (B, 3, N) per-order efficiencies for [given polarization, pure s, pure p];
 *   amps (B, 3, 4, N) = r_s, r_p, t_s, t_p per column or NULL; status (B) WB_ST_* bits.
 * Reference: rcwa/_engine/scattering.py:1185-1456 (_smm_sp, smm_2d) with :907-994
 * (_sp_scattering_result), rcwa/_engine/solve_1d.py:1588-1610 (sp_efficiencies),
 * observations/power.py:13-159. */
int wb_solve_batch(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* conv,
                   const int32_t* layer_index, const double* thickness, const double* wavelength,
                   const double* period, const double* theta, const double* phi,
                   const wb_complex* eps_top, const wb_complex* eps_bot, const wb_complex* pol,
                   double* R, double* T, wb_complex* amps, int32_t* status, int precision,
                   void* stream);

/* Stage C alone: the S-matrix cascade and the efficiencies of B solves from given modes, e.g.
 * eigenpairs kept on the device from earlier wb_layer_modes calls. Every array is a device pointer.
 *   W, V (B*L, 2N, 2N) column-major and q (B*L, 2N) of the (solve, layer) pairs p = b*L + l, as
 *   wb_layer_modes returns them (computed with the order wavevectors of the same wavelength,
 *   period and angles); thickness (B, L); the other arrays as in wb_solve_batch.
 * precision: WB_PRECISION_FP64 (FP64 cascade) or WB_PRECISION_MIXED (FP32 cascade refined against
 * the given modes). Reference: rcwa/_engine/scattering.py:116-200, 1272-1293 (_ab_matrices,
 * _s_layer, redheffer_star, the SMM cascade) and :907-994; solve_2d.py:2584-2616 (sp_modes_2d). */
int wb_smm_solve(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                 const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                 const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                 const wb_complex* pol, double* R, double* T, wb_complex* amps, int32_t* status, int precision,
                 void* stream);

/* Reverse passes (vector-Jacobian products), FP64, on the device. Cotangents follow torch's
 * convention: for a real loss l and a complex z = x + iy the cotangent is dl/dx + i dl/dy (a real
 * input's gradient is its real part). Cotangent inputs marked "or NULL" count as zero. They
 * replace the reference's differentiated backends for this path: rcwa/_engine/modal_gradient.py
 * :56-251 (eigen-solve generator with broadened reciprocal gaps), _common/backend.py:1724-1759
 * (_eig_grad), and torch autograd through scattering.py:116-200, 907-994 and
 * factorization.py:289-671.
 *
 * Reverse of wb_smm_solve (FP64 form): from the cotangents g_R, g_T (device, (B, 3, N), or NULL)
 * of its R and T, the cotangents of its W, V (B*L, 2N, 2N), q (B*L, 2N) and thickness (B, L),
 * all overwritten. The cascade is recomputed with its intermediates, chunked by the handle's
 * budget. Inputs as wb_smm_solve; status (B) gets WB_ST_SINGULAR for a singular factor. */
int wb_smm_solve_vjp(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                     const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                     const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                     const wb_complex* pol, const double* g_R, const double* g_T, wb_complex* g_W, wb_complex* g_V,
                     wb_complex* g_q, double* g_thickness, int32_t* status, void* stream);

/* Reverse of wb_layer_modes: from the cotangents of its outputs w, q (n_pairs, 2N) and W, V
 * (n_pairs, 2N, 2N) (each or NULL), the cotangents g_conv (device, (n_conv, 3, N, N), overwritten)
 * of the slots epx, epy, epz_i, summed over the pairs that read each layer. The other inputs are
 * wb_layer_modes's inputs and outputs. Each mode's scale is a free gauge that no RCWA answer
 * depends on, so the eigenvector cotangent's component along it is dropped; exactly degenerate
 * eigenvalues use the broadened gap conj(d)/(|d|^2 + (2N u max|w|)^2). status (n_pairs) or NULL. */
int wb_layer_modes_vjp(wb_handle* h, int n_pairs, int hu, int hv, int n_conv, const wb_complex* conv,
                       const int32_t* pair_layer, const double* kx, const double* ky, const wb_complex* w,
                       const wb_complex* q, const wb_complex* W, const wb_complex* V, const wb_complex* g_w,
                       const wb_complex* g_q, const wb_complex* g_W, const wb_complex* g_V, wb_complex* g_conv,
                       int32_t* status, void* stream);

/* Reverse of wb_assemble_li (sampled coefficients, fixed nesting): from the cotangents of the
 * slots (device, each (L, N, N) column-major, or NULL) the cotangent g_eps (device, (L, ny, nx),
 * overwritten) of the rasters. eps is the forward's input, epx and epz_i its outputs (their
 * inverses' reverse needs them). status (1) or NULL. */
int wb_assemble_li_vjp(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                       const wb_complex* epx, const wb_complex* epz_i, const wb_complex* g_epx,
                       const wb_complex* g_epy, const wb_complex* g_epz_i, wb_complex* g_eps, int32_t* status,
                       void* stream);

/* The stack's scattering matrix at its two half-space ports, as the reference publishes it
 * (Outputs(scattering=True), result.scattering), from given modes (FP64). Inputs as wb_smm_solve
 * without pol. Outputs (device, each (B, 2N, 2N) column-major): S11 reflection back into the
 * superstrate, S12 transmission from the substrate into the superstrate, S21 transmission from
 * the superstrate into the substrate, S22 reflection back into the substrate. Rows and columns
 * are the s amplitudes of the N orders followed by the p port variables (the p wave's magnetic
 * field: S11 applied to a unit s column is r_s, to a unit p column -r_p), every order referenced
 * at the cell centre. Reference: rcwa/_engine/scattering.py:482-605 (ScatteringMatrix,
 * _scattering_matrix), :1272-1293 (the cascade that forms it). */
int wb_scattering_matrix(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                         const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                         const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                         wb_complex* S11, wb_complex* S12, wb_complex* S21, wb_complex* S22, int32_t* status,
                         void* stream);

/* The ETM connecting algorithm (Numerics(algorithm='etm')) from given modes, FP64: the enhanced
 * transmittance matrix recursion bottom-up and the final matching at the superstrate. Inputs and
 * outputs as wb_smm_solve (FP64 form). Reference: rcwa/_engine/solve_2d.py:2619-2843 (the 2D ETM
 * path), solve_1d.py:1389-1520 (final_matching). */
int wb_etm_solve(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                 const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                 const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                 const wb_complex* pol, double* R, double* T, wb_complex* amps, int32_t* status, void* stream);

/* Every layer's mode amplitudes inside the stack, for the field reconstruction, from given modes
 * (FP64). Inputs as wb_smm_solve without pol, plus C (device, (B, 2N, k) column-major per solve):
 * k incidence columns in the superstrate's port variables. Outputs (device): plus, minus_top,
 * minus_bottom (B, L, 2N, k): each layer's down-going amplitudes at its top face and its up-going
 * ones at its top and bottom faces, in the layer's s/p-rotated mode basis; cref, ctrn (B, 2N, k):
 * the reflected and transmitted columns in the half-space port variables. Reference:
 * rcwa/_engine/scattering.py:236-350 (_below_reflections, _field_state). */
int wb_layer_amplitudes(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                        const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                        const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                        const wb_complex* C, int k, wb_complex* plus, wb_complex* minus_top, wb_complex* minus_bottom,
                        wb_complex* cref, wb_complex* ctrn, int32_t* status, void* stream);

/* The same solve from HOST buffers: rasters in, efficiencies out. Copies inputs to the
 * device, assembles the L layers (stage A), solves the B problems, copies R, T and status
 * back and synchronises. eps: host (L, ny, nx); the other arrays as in wb_solve_batch but in
 * host memory (pinned memory makes the copies asynchronous DMA). The device block that stages
 * inputs, slots and outputs belongs to the handle: allocated by the first call, grown only when
 * a later call needs more, freed by wb_destroy. Reference: the rcwa.run(problem) lifecycle,
 * rcwa/_lifecycle.py:698-803. */
int wb_solve_host(wb_handle* h, int B, int L, int ny, int nx, int hu, int hv,
                  const wb_complex* eps, const int32_t* layer_index, const double* thickness,
                  const double* wavelength, const double* period, const double* theta,
                  const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                  const wb_complex* pol, double* R, double* T, int32_t* status, int precision);

/* Bytes of arena one chunk of `chunk` solves with L layers and N orders needs (FP64 form). */
size_t wb_solve_workspace_bytes(int hu, int hv, int L, int chunk);

/* The same for any WB_PRECISION_* form (the mixed forms keep FP32 copies, group slots and
 * refinement vectors beside the FP64-sized buffers); 0 for invalid arguments. Admission code
 * (the reference's rcwa.check estimates, _lifecycle.py:422-457) sizes batches with it. */
size_t wb_workspace_bytes(int hu, int hv, int L, int chunk, int precision);

/* Stage A without any allocation, for callers that may not allocate device memory (code running
 * inside another component's CUDA-graph capture, servers and plugins whose host owns the device
 * pool, allocation-free real-time paths). No counterpart in the reference. Same inputs and outputs
 * as wb_assemble_li, no handle: scratch lives in a fixed 32 MiB device array of the library
 * (wb_assemble_li_noalloc_limit() bytes), held by every GPU that loads it until exit. Layers are
 * assembled one at a time, so the limit is per layer; a layer that needs more scratch is refused
 * with WB_E_INVALID before any GPU work. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current, so make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race and must be ordered by the caller.
 * status: device int32 (1) or NULL, not cleared here. */
int wb_assemble_li_noalloc(const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                           wb_complex* epx, wb_complex* epy, wb_complex* epz_i, int32_t* status,
                           void* stream);
size_t wb_assemble_li_noalloc_limit(void);

/* Number of kernels the library has launched in this process since it was loaded, over all
 * handles (for accounting: take differences around a region). The handle is not consulted. */
long long wb_kernel_launches(wb_handle* h);

/* Launch-shape tunables, process-wide: 0 restores the library's own choice. The autotuner
 * (wavebit_gb300/autotune.py) times candidates per (orders, layers, batch) bucket and sets them
 * before each batch. Thread counts never change a result; WB_TUNE_TENSOR_CORES = 1 moves the FP32
 * complex products from the tensor cores (split TF32) to FP32 SIMT, which changes their rounding
 * within FP32 accuracy. No counterpart in the reference (its backends leave launch shapes to
 * LAPACK and torch). */
#define WB_TUNE_QR_THREADS 0     /* threads of a QR-sweep CTA (64..1024, multiple of 32) */
#define WB_TUNE_HRD_THREADS 1    /* threads of a Hessenberg-reduction CTA (64..1024, multiple of 32) */
#define WB_TUNE_LU_THREADS 2     /* reserved: threads of an LU / triangular-solve CTA */
#define WB_TUNE_TENSOR_CORES 3   /* 1: FP32 complex products on the SIMT kernel instead of tcgen05 */
#define WB_TUNE_HRD_BLOCKED 4    /* 1: the FP32 Hessenberg reduction one column at a time instead of in panels */
#define WB_TUNE_COUNT 8
int wb_set_tuning(int key, int value);
/* The current value of a tunable (0 = the library's own choice), or -1 for an unknown key. */
int wb_get_tuning(int key);

/* CTAs of the tensor-core complex product (tcgen05, 3xTF32) whose bounded wait on their own
 * MMAs ran out since the library was loaded (they skip their output and raise this count); 0 in
 * a healthy run, -1 if the counter cannot be read. No counterpart in the reference. */
long long wb_tensor_core_errors(void);

/* Live timing of the Schur-form QR sweeps, the eigen-solve's dominant kernel, for measurement:
 * while enabled, CUDA events are recorded on the launching stream around every sweep launch.
 * wb_profile_qr(1) clears and enables, wb_profile_qr(0) clears and disables. wb_profile_qr_read
 * gives, for real type 0 (FP64), 1 (FP32) or 2 (double-float), the summed event time in ms, the
 * number of launches and their algorithmic bytes (every bulge step moves each of its 2n - 2
 * element pairs' moving element once, in and out). It synchronises on the recorded events. No
 * counterpart in the reference. */
int wb_profile_qr(int enable);
int wb_profile_qr_read(int real_type, double* ms, long long* launches, double* bytes);

#ifdef __cplusplus
}
#endif
#endif
