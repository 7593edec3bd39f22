/*
 * et_array_interface.h -- C-ABI of lib_et_array_interface.so, the GB300
 * (sm_103a) implementation of NiftyRec's rotation-based SPECT emission path.
 *
 * Every entry point of the reference's emission array interface on this path
 * keeps its name, argument list, argument meaning and status codes; each
 * declaration names the reference declaration it replaces.  Buffers are
 * caller-owned host float32 arrays in nifti order (size[0] fastest); outputs
 * are written in place; calls are synchronous.  The computation always runs on
 * the GPU: the "Gpu"/"GPU"/"use_gpu" flags are accepted and ignored.
 *
 * Status codes (emission-lib/_et_common.h:40-48): 0 success, 1 unspecified,
 * 2 parameters, 3 kernel, 4 allocgpu, 5 alloccpu, 6 transfergpu,
 * 7 nogpubuilt, 8 nogpuinstalled; 10 (new) the problem does not fit the fixed
 * scratch of nrgb_backproject_device_noalloc.  9 is not used.
 */
#ifndef NIFTYREC_GB300_ET_ARRAY_INTERFACE_H
#define NIFTYREC_GB300_ET_ARRAY_INTERFACE_H

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* SimpleWrap status helpers -- emission-lib/_et_array_interface.h:22-27. */
int status_success(int *status);
int status_io_error(int *status);
int status_initialisation_error(int *status);
int status_parameter_error(int *status);
int status_unhandled_error(int *status);
int echo(int *in, int *out);

/* Message of a status code -- emission-lib/_et_common.h:56. */
char *niftyrec_error_msg(int status);

/* Devices -- emission-lib/_et_array_interface.h:36-41. */
int et_array_list_gpus(int *gpu_count, int *gpus_info_array);
int et_array_set_gpu(int id);
int et_array_set_gpu_pointer(int *id);
int et_array_isinstalled(void);
int et_array_reset_gpu(void);
unsigned short et_array_is_block_multiple(unsigned short size);
unsigned short et_array_get_block_size(void);

/* Projection -- emission-lib/_et_array_interface.h:44 (scalars by pointer). */
int SPECT_project_parallelholes(float *activity, int *activity_size, float *sinogram, int *sinogram_size,
                                float *cameras, int *cameras_size, float *psf, int *psf_size, float *attenuation,
                                int *attenuation_size, float *Background, float *Background_attenuation, int *Gpu,
                                int *Truncate_negative_values);

/* Backprojection -- emission-lib/_et_array_interface.h:45. */
int SPECT_backproject_parallelholes(float *sino, int *sino_size, float *bkpr, int *bkpr_size, float *cameras,
                                    int *cameras_size, float *psf, int *psf_size, float *attenuation,
                                    int *attenuation_size, float *Background, float *Background_attenuation,
                                    int *Gpu, int *Truncate_negative_values);

/* By-value spellings bound by Python/NiftyRec/NiftyRec/NiftyRec.py:83-84 and
 * :145-146 (absent from the reference library itself). */
int et_array_project(float *activity, int *activity_size, float *sinogram, int *sinogram_size, float *cameras,
                     int *cameras_size, float *psf, int *psf_size, float *attenuation, int *attenuation_size,
                     float background, float background_attenuation, int gpu, int truncate_negative_values);
int et_array_backproject(float *sino, int *sino_size, float *bkpr, int *bkpr_size, float *cameras,
                         int *cameras_size, float *psf, int *psf_size, float *attenuation, int *attenuation_size,
                         float background, float background_attenuation, int gpu, int truncate_negative_values);

/* Attenuation gradient -- emission-lib/_et_array_interface.h:48 (the GPU
 * semantics of emission-lib/_et.cpp:1679-1924); et_array_attenuation_gradient
 * is the same function under the spelling of the project description. */
int et_array_gradient_attenuation(float *sino, int *sino_size, float *activity, int *activity_size,
                                  float *gradient, int *gradient_size, float *cameras, int *cameras_size, float *psf,
                                  int *psf_size, float *attenuation, int *attenuation_size, float background,
                                  float background_attenuation, int GPU, int truncate_negative_values);
int et_array_attenuation_gradient(float *sino, int *sino_size, float *activity, int *activity_size,
                                  float *gradient, int *gradient_size, float *cameras, int *cameras_size, float *psf,
                                  int *psf_size, float *attenuation, int *attenuation_size, float background,
                                  float background_attenuation, int GPU, int truncate_negative_values);

/* Projection with partial sums -- emission-lib/_et_array_interface.h:47
 * (GPU semantics of et_project_partial_gpu, emission-lib/_et.cpp:2106-2436;
 * the reference's CPU path is a stub).  Per camera: the projection, and in
 * partialsum ([nx, ny, nz, n_cameras]) the emission reaching each depth from
 * the far side, in the rotated frame or, with do_rotate_partial, rotated back
 * to the image frame.  background_image ([nx, ny]) scales the background or
 * is NULL. */
int et_array_project_partial(float *activity, int *activity_size, float *sinogram, int *sinogram_size,
                             float *partialsum, int *partialsum_size, float *cameras, int *cameras_size, float *psf,
                             int *psf_size, float *attenuation, int *attenuation_size, float background,
                             float *background_image, float background_attenuation, int GPU,
                             int truncate_negative_values, int do_rotate_partial);

/* Fisher information of a grid of points -- emission-lib/_et_array_interface.h:50-51
 * (et_fisher_grid, emission-lib/_et.cpp:531-746).  grid_ptr: a volume with
 * values 1..n at the n grid points (n = fisher_size[0]), 0 elsewhere;
 * fisher_ptr / fisher_prior_ptr: [n, n] outputs (the prior may be NULL).  The
 * first form projects the activity; the second takes a projection
 * (sinogram_size) and the grid volume's size (bkpr_size).  epsilon is unused,
 * as in the reference.  A PSF is required. */
int et_array_fisher_grid(float *activity_ptr, int *activity_size, float *cameras, int *cameras_size, float *psf,
                         int *psf_size, float *grid_ptr, float *fisher_ptr, float *fisher_prior_ptr, int *fisher_size,
                         float *attenuation, int *attenuation_size, float epsilon, float background,
                         float background_attenuation, int GPU);
int et_array_fisher_grid_projection(float *sinogram_ptr, int *sinogram_size, int *bkpr_size, float *cameras,
                                    int *cameras_size, float *psf, int *psf_size, float *grid_ptr, float *fisher_ptr,
                                    float *fisher_prior_ptr, int *fisher_size, float *attenuation,
                                    int *attenuation_size, float epsilon, float background,
                                    float background_attenuation, int GPU);

/* PSF / camera helpers -- emission-lib/_et_array_interface.h:53-55. */
int et_array_calculate_size_psf(unsigned int *psf_size_x, unsigned int *psf_size_y, float fwhm_pixels_dist0,
                                float sensitivity0, float dist0, float fwhm_pixels_dist1, float sensitivity1,
                                float dist1);
int et_array_make_psf(float *psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float fwhm_pixels_dist0,
                      float sensitivity0, float dist0, float fwhm_pixels_dist1, float sensitivity1, float dist1,
                      unsigned int N_psf_planes);
int et_array_make_cameras(float *cameras_data, float firstcamera_deg, float lastcamera_deg, unsigned int n_cameras,
                          unsigned int rotation_axis);

/* Affine transformation of a volume -- emission-lib/_et_array_interface.h:31.
 * out(x) = trilinear(image, A x), `background` outside; A = affine_ptr, 4 x 4
 * in column-major order (affine_size {4, 4}); the output has image_size.  The
 * reference ignores affine_ptr (a zeroed matrix, FIXME in its source); this
 * applies it, as documented. */
int et_array_affine(float *image_ptr, int *image_size, float *transformed_image_ptr, int *transformed_image_size,
                    float *affine_ptr, int *affine_size, float background, int GPU);

/* Per-slice 2D convolution -- emission-lib/_et_array_interface.h:33.
 * image [nx, ny, nz] (x fastest), kernel slices psf [kx, ky, nz] (odd kx, ky),
 * out(x, y, z) = sum_{i,j} psf(i, j, z) image(x + (kx-1)/2 - i, y + (ky-1)/2 - j, z)
 * with the image clamped to its border, as the reference's FFT path intends
 * (its CPU path is a stub returning 1, its GPU path shifts the size array);
 * out has the image's size. */
int et_array_convolve(float *image, int *image_size, float *out, int *out_size, float *psf, int *psf_size, int GPU);

/* Rotation of a volume -- emission-lib/_et_array_interface.h:32. */
int et_array_rotate(float *image, int *size, float *rotated_image, float *angles, float *centers, float background,
                    int axis_order, int GPU);

/* OSEM / MLEM -- emission-lib/_et_array_interface.h:56-59. */
int et_array_osem(float *activity_data, unsigned int size_x, unsigned int size_y, unsigned int subset_order,
                  float *sinogram_data, int n_cameras, float firstcamera, float lastcamera,
                  unsigned int rotation_axis, int iterations, int use_attenuation, float *attenuation_data,
                  int use_psf, float *psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float background,
                  float background_attenuation, float epsilon, int use_gpu);
int et_array_osem_step(float *activity_data, int size_x, int size_y, unsigned int subset_order,
                       float *sinogram_data, int n_cameras, float *cameras_data, int use_attenuation,
                       float *attenuation_data, int use_psf, float *psf_data, unsigned int psf_size_x,
                       unsigned int psf_size_y, float background, float background_attenuation, float epsilon,
                       int use_gpu);
int et_array_mlem(float *activity_data, unsigned int size_x, unsigned int size_y, float *sinogram_data,
                  int n_cameras, float firstcamera, float lastcamera, unsigned int rotation_axis, int iterations,
                  int use_attenuation, float *attenuation_data, int use_psf, float *psf_data,
                  unsigned int psf_size_x, unsigned int psf_size_y, float background, float background_attenuation,
                  float epsilon, int use_gpu);
int et_array_mlem_step(float *activity_data, int size_x, int size_y, float *sinogram_data, int n_cameras,
                       float *cameras_data, int use_attenuation, float *attenuation_data, int use_psf,
                       float *psf_data, unsigned int psf_size_x, unsigned int psf_size_y, float background,
                       float background_attenuation, float epsilon, int use_gpu);

/* Deterministic OSEM step over explicit camera indexes.  Replaces the random
 * subset draw of et_array_osem_step (emission-lib/_et_array_interface.cpp:1001-1009,
 * unseeded rand()) so that results are reproducible. */
int et_array_osem_step_subset(float *activity_data, int size_x, int size_y, float *sinogram_data, int n_cameras,
                              float *cameras_data, const int *camera_indexes, int n_subset, int use_attenuation,
                              float *attenuation_data, int use_psf, float *psf_data, unsigned int psf_size_x,
                              unsigned int psf_size_y, float background, float background_attenuation,
                              float epsilon);

/* Device-pointer entry points (additions; the reference's GPU path has no
 * equivalent -- it copies host buffers in and out on every call,
 * emission-lib/_et.cpp:917-1137).  Buffers are device float32 in nifti order;
 * cameras and PSF are host arrays; work is enqueued on `stream` (a
 * cudaStream_t) and the call returns without waiting.  size = {nx, ny, nz}.
 * For the backprojection the centre of rotation is (size0, size1, size0),
 * as in SPECT_backproject_parallelholes; mode 0 is the reference backprojector
 * (inverse-rotation gather), mode 1 the exact transpose of the projector for
 * the given mu (transposed PSF and bilinear weights; backgrounds do not enter:
 * they are constants of the projector), used for gradients. */
int nrgb_project_device(const float *d_activity, const float *d_attenuation, const int *size, float *d_sinogram,
                        const float *cameras, const int *cameras_size, const float *psf, const int *psf_size,
                        float background, float background_attenuation, int truncate, void *stream);
int nrgb_backproject_device(const float *d_sinogram, const float *d_attenuation, const int *size, float *d_out,
                            const float *cameras, const int *cameras_size, const float *psf, const int *psf_size,
                            float background, float background_attenuation, int truncate, int mode, void *stream);

/* bfloat16 storage (additions; the reference is float32 throughout):
 * d_activity and d_attenuation are device bfloat16 volumes in nifti order;
 * every product and sum is float32, the depth sums of the fused kernels
 * (transmission prefix, projection) are Kahan-compensated, and sinograms and
 * backprojections are float32.  Same arguments and status codes as the
 * float32 entry points above. */
int nrgb_project_device_bf16(const void *d_activity, const void *d_attenuation, const int *size, float *d_sinogram,
                             const float *cameras, const int *cameras_size, const float *psf, const int *psf_size,
                             float background, float background_attenuation, int truncate, void *stream);
int nrgb_backproject_device_bf16(const float *d_sinogram, const void *d_attenuation, const int *size, float *d_out,
                                 const float *cameras, const int *cameras_size, const float *psf, const int *psf_size,
                                 float background, float background_attenuation, int truncate, int mode,
                                 void *stream);

/* float64 reference run (additions): the reference projector and
 * backprojector (general-orientation kernels in the reference's operation
 * order) with positions, weights, PSF, exp and every sum in double, on device
 * double buffers in nifti order.  Cameras and PSF are the float32 host arrays
 * of the float32 entry points, widened exactly.  The float32 and bfloat16
 * results are measured against this run.  Slow (float64 throughput), for
 * error reports only. */
int nrgb_project_device_f64(const double *d_activity, const double *d_attenuation, const int *size,
                            double *d_sinogram, const float *cameras, const int *cameras_size, const float *psf,
                            const int *psf_size, double background, double background_attenuation, int truncate,
                            void *stream);
int nrgb_backproject_device_f64(const double *d_sinogram, const double *d_attenuation, const int *size,
                                double *d_out, const float *cameras, const int *cameras_size, const float *psf,
                                const int *psf_size, double background, double background_attenuation, int truncate,
                                void *stream);
int nrgb_osem_ratio_device_f64(const double *d_counts, double *d_projection, long long n, double epsilon,
                               void *stream);
int nrgb_osem_update_device_f64(double *d_activity, const double *d_numerator, const double *d_denominator,
                                long long n, double epsilon, void *stream);

/* Exact gradient with respect to mu of sum(g * P(activity, mu)), P the
 * projector without truncation, g = d_grad_sinogram (device, nifti order):
 * dP/dmu_z' = -(sum_{z >= z'} PSF(rotated activity)_z exp(-T_z) + bg exp(-T_N))
 * in the rotated frame, mapped back by the transposed trilinear weights.  No
 * counterpart in the reference: its et_array_gradient_attenuation
 * (emission-lib/_et.cpp:1679-1924) ignores the PSF coupling, the sign and the
 * background; that function is kept above with the reference's semantics. */
int nrgb_attenuation_grad_device(const float *d_grad_sinogram, const float *d_activity, const float *d_attenuation,
                                 const int *size, float *d_out, const float *cameras, const int *cameras_size,
                                 const float *psf, const int *psf_size, float background,
                                 float background_attenuation, void *stream);

/* et_array_gradient_attenuation (emission-lib/_et_array_interface.h:48, the
 * GPU semantics of emission-lib/_et.cpp:1679-1924) on device buffers in nifti
 * order, enqueued on `stream` (a cudaStream_t or null): size = {nx, ny, nz},
 * d_sinogram [ncam][ny][nx].  No counterpart in the reference (which takes
 * host arrays only). */
int nrgb_gradient_attenuation_device(const float *d_sinogram, const float *d_activity, const float *d_attenuation,
                                     const int *size, float *d_out, const float *cameras, const int *cameras_size,
                                     const float *psf, const int *psf_size, float background,
                                     float background_attenuation, int truncate, void *stream);

/* Projection and backprojection in one call (addition; the sequence the
 * reference's et_array_osem_step / et_array_mlem_step run inside one step,
 * emission-lib/_et_array_interface.cpp:1017-1035, of the et_project /
 * et_backproject pair emission-lib/_et.cpp:122 and :312).  Projects
 * d_activity into d_sinogram exactly as nrgb_project_device, then backprojects
 * d_backproject_input -- or, when it is null, the projection just written --
 * into d_backprojection exactly as nrgb_backproject_device (mode 0 reference,
 * 1 exact transpose), with the same cameras, PSF, mu, backgrounds and
 * truncation.  For cameras about the gantry axis the volumes are laid out
 * once for both halves, the projector leaves the backprojector's
 * transmission carries (per depth slab mu prefix sums) and the projection
 * feeds the backprojector without another layout pass; results equal the two
 * calls' within float32 rounding.  Device buffers in nifti order; returns once
 * the work is enqueued on `stream`. */
int nrgb_project_backproject_device(const float *d_activity, const float *d_attenuation, const int *size,
                                    float *d_sinogram, const float *d_backproject_input, float *d_backprojection,
                                    const float *cameras, const int *cameras_size, const float *psf,
                                    const int *psf_size, float background, float background_attenuation,
                                    int truncate, int mode, void *stream);

/* The same with bfloat16 activity and mu (nifti order; float32 sinograms and
 * backprojection), as nrgb_project_device_bf16 / nrgb_backproject_device_bf16
 * (addition; no counterpart in the reference). */
int nrgb_project_backproject_device_bf16(const void *d_activity, const void *d_attenuation, const int *size,
                                         float *d_sinogram, const float *d_backproject_input, float *d_backprojection,
                                         const float *cameras, const int *cameras_size, const float *psf,
                                         const int *psf_size, float background, float background_attenuation,
                                         int truncate, int mode, void *stream);

/* Backprojection that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: a plug-in inside a host
 * application whose framework allocator already holds the GPU's memory (a
 * cudaMalloc there fails or forces the host to free its cache), or a
 * real-time reconstruction loop that must not enter the driver's allocator
 * (unbounded latency, possible device-wide synchronisation).  Same arguments
 * and result (within float32 rounding) as nrgb_backproject_device with mode 0;
 * cameras about the gantry axis y run the same fused kernels, every other
 * camera (also cameras about x, which nrgb_backproject_device serves with the
 * fused kernels) runs the general-orientation kernels.  Every temporary lives
 * in a fixed 64 MiB __device__ array of this library (held by every GPU that
 * loads it, until the process exits); camera matrices and the separated PSF
 * are stored into it by kernels that carry them in their launch parameters.
 * Problems whose work space does not fit (e.g. 128^3 x 120 cameras) return
 * status 10; use nrgb_backproject_device for those.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress), once per
 * device with that device current; make that first call before any stream
 * capture.  All calls share the array and it keeps the last call's contents
 * (every call overwrites what it reads); calls that overlap on the GPU (two
 * streams, two threads) race on it, so serialise them.  No cudaMalloc,
 * cudaFree or allocating library routine is called (with the launch profiler
 * off, its default). */
int nrgb_backproject_device_noalloc(const float *d_sinogram, const float *d_attenuation, const int *size,
                                    float *d_out, const float *cameras, const int *cameras_size, const float *psf,
                                    const int *psf_size, float background, float background_attenuation,
                                    int truncate, void *stream);

/* The elementwise stages of et_array_osem_step on device buffers (additions;
 * emission-lib/_et_array_interface.cpp:1022-1028 and :1036-1044 run them on
 * host arrays inside the step).  ratio overwrites d_projection with
 * y / p (y / epsilon where p < epsilon); update does
 * activity *= numerator / max(denominator, epsilon).  For callers that build
 * the step from partial backprojections, e.g. summed across processes that
 * each own a share of a subset's cameras. */
int nrgb_osem_ratio_device(const float *d_counts, float *d_projection, long long n, float epsilon, void *stream);
int nrgb_osem_update_device(float *d_activity, const float *d_numerator, const float *d_denominator, long long n,
                            float epsilon, void *stream);

/* Host-side fault injection (no counterpart in the reference): the next n
 * device work-space allocations that would grow the library's arena fail with
 * status 4 (allocgpu) before any CUDA call is made, so callers' error paths
 * can be tested without a GPU fault.  n = 0 clears it. */
int nrgb_debug_fail_allocations(int n);

/* Diagnostics: 1 if the calling thread's last call ran the fused y-gantry
 * kernels, 2 if it ran the general-orientation kernels, 0 before any call. */
int nrgb_last_path(void);

/* Plans (no counterpart in the reference, whose OSEM step re-uploads and
 * recomputes everything per call, emission-lib/_et_array_interface.cpp:972-1131).
 * A plan holds device state for one grid, camera set, PSF and attenuation map:
 * camera matrices, mu in column layout, the transmission carries of every
 * camera and, after nrgb_plan_osem_prepare, the per-subset sensitivity images.
 * nrgb_plan_create allocates (and computes) everything; the execute calls
 * (project, backproject, osem_step) allocate nothing and copy nothing from the
 * host, so a sequence of them can be captured in a CUDA graph.  layout: 0 =
 * nifti order, 1 = column layout [planes][nx][round_up(ny,4)] with zero pads
 * (fused plans only; convert with nrgb_layout_convert).  Sinograms of a subset
 * hold its cameras in nrgb_plan_subset_cameras order.  The projection uses the
 * centre rule of SPECT_project_parallelholes, the backprojection the rule of
 * SPECT_backproject_parallelholes. */
int nrgb_plan_create(void **out_plan, const int *size, const float *cameras, const int *cameras_size,
                     const float *psf, const int *psf_size, const float *d_attenuation, float background,
                     float background_attenuation, const int *subset_of_camera, int n_subsets, void *stream);
int nrgb_plan_destroy(void *plan);
int nrgb_plan_shape(void *plan, int *out);
int nrgb_plan_subset_cameras(void *plan, int subset, int *idx_out);
int nrgb_plan_project(void *plan, int subset, const float *d_activity, float *d_sinogram, int layout,
                      int truncate, void *stream);
int nrgb_plan_backproject(void *plan, int subset, const float *d_sinogram, float *d_out, int layout,
                          int truncate, void *stream);
int nrgb_plan_osem_prepare(void *plan, int layout, void *stream);
int nrgb_plan_osem_step(void *plan, int subset, float *d_activity, const float *d_counts, float epsilon,
                        void *stream);
int nrgb_layout_convert(const float *src, float *dst, int nx, int ny, int planes, int direction, int truncate,
                        void *stream);
/* One-step-late MAP-EM step with the quadratic MRF prior on a plan (the
 * reference runs it in Python on host arrays: et_osmapem_step,
 * Python/NiftyRec/NiftyRec/NiftyRec.py:224-245, prior gradient :400-404).  The
 * prior gradient (26 x minus the 26 neighbours, zero outside the grid) is
 * computed from the current activity; x *= max(A^T(y / (max(Ax, 0) + eps)), 0)
 * / (max(sens - beta g, 0) + eps).  Layouts as nrgb_plan_osem_step. */
int nrgb_plan_osmapem_step(void *plan, int subset, float *d_activity, const float *d_counts, float beta,
                           float epsilon, void *stream);
/* The prior gradient alone, device volume in nifti order; size = {nx, ny, nz}. */
int nrgb_mrf_gradient_device(const float *d_activity, float *d_gradient, const int *size, void *stream);

/* Batches (no counterpart in the reference): one OSEM subset step of up to 64
 * plans at once -- a persistent projector launch whose clusters take
 * (volume, row window, camera, x-tile) work items from a queue, one ratio
 * launch, each plan's backprojection, one update launch.  Plans must be fused
 * and prepared for OSEM in column layout (nrgb_plan_osem_prepare(plan, 1)).
 * The batch owns each volume's activity and counts (column layout); set them
 * with nrgb_batch_set_activity / nrgb_batch_set_counts (device nifti arrays,
 * counts in original camera order) and read the activity back with
 * nrgb_batch_get_activity.  nrgb_batch_osem_step allocates nothing and copies
 * nothing from the host, so steps can be captured in a CUDA graph; volume v
 * runs subset (step mod n_subsets_v), and with iterations > 0 sits out steps
 * >= iterations * n_subsets_v. */
int nrgb_batch_create(void **out_batch, void *const *plans, int n_plans, void *stream);
int nrgb_batch_destroy(void *batch);
int nrgb_batch_set_counts(void *batch, int volume, const float *d_counts, void *stream);
int nrgb_batch_set_activity(void *batch, int volume, const float *d_activity, void *stream);
int nrgb_batch_get_activity(void *batch, int volume, float *d_activity, void *stream);
int nrgb_batch_osem_step(void *batch, int step, int iterations, float epsilon, void *stream);

/* Tuning table of the fused backprojector (no counterpart in the reference):
 * cameras per L2-resident scratch group for a problem shape (nx, ny, nz,
 * n_cameras); an all-zero shape sets the default for shapes without an entry
 * (none initially: then even groups of at most 48 cameras, at most 2 GiB of
 * scratch each); group 0 removes the entry.  niftyrec_gb300.autotune measures
 * candidates and records the fastest. */
int nrgb_set_backproject_group(int nx, int ny, int nz, int ncam, int group);
int nrgb_get_backproject_group(int nx, int ny, int nz, int ncam);
/* Tuning table of the fused projector (no counterpart in the reference):
 * depth slabs per (camera, x-tile) item -- the thread-block cluster size, 2,
 * 4, 8 or 16 (a non-portable cluster size: 8 where it cannot be resident) --
 * for a problem shape; 0 (the initial state) lets the launcher take the
 * fewest slabs that give four waves of thread blocks.
 * niftyrec_gb300.autotune measures the candidates and records the fastest. */
int nrgb_set_project_slabs(int nx, int ny, int nz, int ncam, int slabs);
int nrgb_get_project_slabs(int nx, int ny, int nz, int ncam);
/* Mirror cameras (no counterpart in the reference).  Two gantry cameras at
 * opposite angles (difference pi within 1e-6 rad) about the grid centre
 * sample the same points: the second one's rotated volume is the first one's
 * mirrored in x and z.  With on = 1 (the default) the fused projector serves
 * such a pair from one set of bilinear samples (the second camera's sampling
 * positions are the first one's, mirrored, instead of those of its own float
 * matrix: a difference below 1e-6 of the projection); 0 computes every camera
 * from its own matrix, as the reference.  Applies to calls made afterwards. */
int nrgb_set_mirror_pairs(int on);
int nrgb_get_mirror_pairs(void);
/* Deterministic gradients (no counterpart in the reference).  With on = 1 the
 * exact-transpose backprojector (back_mode 1) and the exact d/dmu
 * (nrgb_attenuation_grad_device) on the fused gantry kernels write their
 * rotated-frame values into camera-group scratch volumes and sum them with a
 * transposed bilinear gather in a fixed order, so repeated calls give
 * bit-identical results; 0 (the default) scatters with vector reductions
 * (faster, summation order varies between runs at the float rounding level).
 * Cameras off the gantry forms keep the atomic trilinear scatter of the
 * general path.  The reference-mode backprojector, the projector and the
 * OSEM/MLEM steps are deterministic either way.  Applies to calls made
 * afterwards (and to plans made afterwards). */
int nrgb_set_deterministic(int on);
int nrgb_get_deterministic(void);
/* Host-side introspection (no counterpart in the reference; no GPU needed).
 * nrgb_mirror_units: the {camera, mate} pairs (mate -1 when unpaired) the
 * fused kernels form for this camera table and volume size {nx, ny, nz};
 * *n_units = 0 when every camera runs on its own.  nrgb_row_windows: the row
 * windows {first row, rows, first valid row, end of valid rows} of ny rows for
 * a PSF of width psf_k (0: none).  Both return status 2 when the output
 * cannot hold the result (the count is still written). */
int nrgb_mirror_units(const float *cameras, const int *cameras_size, const int *size, int *out_units, int max_units,
                      int *n_units);
int nrgb_row_windows(int ny, int psf_k, int *out, int max_windows, int *n_windows);

/* Instrumentation (no counterpart in the reference).  nrgb_launch_count: CUDA
 * kernels this library launched since it was loaded.  nrgb_profile_enable(1)
 * brackets every launch with CUDA events on its stream (0 turns it off; both
 * clear the record); nrgb_profile_summary writes one "name launches total_ms"
 * line per kernel into buf, waiting for the recorded events, and returns the
 * size it needs.  nrgb_profile_only(name) restricts the timing to launches of
 * that kernel name (null or "" times every launch): the events between
 * launches cost a few microseconds each on the GPU, so a throughput run times
 * one kernel only. */
long long nrgb_launch_count(void);
int nrgb_profile_enable(int on);
int nrgb_profile_summary(char *buf, int len);
int nrgb_profile_only(const char *name);

/* NIfTI-1 single-file images (no counterpart in the reference library; its
 * command-line tool reads and writes them with nifti1_io, apps/command_line_tools/
 * rec_spect.cpp:447-606).  .nii.gz needs zlib at build time
 * (nrgb_nifti_gzip_supported).  nrgb_nifti_info: dims = {ndim, dim1..dim7};
 * nrgb_nifti_read: every voxel as float32 (integer and real datatypes, either
 * byte order, scl_slope applied), n_voxels must match; nrgb_nifti_write:
 * float32 image of dims = {ndim, dim1..dimN}.  Status 2 on any failure. */
int nrgb_nifti_info(const char *path, int *dims);
int nrgb_nifti_read(const char *path, float *data, long long n_voxels);
int nrgb_nifti_write(const char *path, const float *data, const int *dims);
int nrgb_nifti_gzip_supported(void);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif


#ifdef __cplusplus
}
#endif

#endif
