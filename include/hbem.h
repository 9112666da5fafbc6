/*
 * hbem.h -- C ABI of the GB300 HelmholtzBEM assembly-and-resonance path.
 *
 * Plain C: opaque handles, pointers and sizes, int status codes, no exceptions
 * and no C++ / torch types.  Complex matrices are column-major arrays of
 * interleaved (re, im) doubles, the layout of Eigen::MatrixXcd.  Unless a name
 * ends in _device, pointers are host pointers and the call copies.
 *
 * Each entry point names the reference interface it replaces
 * (paths inside marohnicluka/HelmholtzBEM).  Handles are not thread-safe: use
 * one handle per host thread; every handle owns one CUDA stream.
 */
#ifndef HBEM_H
#define HBEM_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
    HBEM_OK = 0,
    HBEM_ERR_INVALID = 1,      /* bad argument (the reference throws std::runtime_error / out_of_range) */
    HBEM_ERR_CUDA = 2,         /* CUDA runtime error */
    HBEM_ERR_NOMEM = 3,        /* device allocation failed */
    HBEM_ERR_NOCONV = 4,       /* an iteration hit its cap (Jacobi sweeps, Newton) */
    HBEM_ERR_SINGULAR = 5,     /* zero pivot */
    HBEM_ERR_NONFINITE = 6,    /* NaN / Inf in a result */
    HBEM_ERR_UNSUPPORTED = 7   /* combination not provided by this build */
};

/* LayerType (include/galerkin_builder.hpp:100-115) */
enum { HBEM_LAYER_DOUBLE = 1, HBEM_LAYER_SINGLE = 2, HBEM_LAYER_HYPERSINGULAR = 4, HBEM_LAYER_ALL = 7 };

/* panel kinds: ParametrizedLine (include/parametrized_line.hpp), ParametrizedCircularArc
 * (include/parametrized_circular_arc.hpp).  5 doubles per panel:
 *   line: x1 y1 x2 y2 (unused)      arc: cx cy r phi_start phi_end                    */
enum { HBEM_PANEL_LINE = 0, HBEM_PANEL_ARC = 1 };

/* BEM spaces by local shape-function count: ContinuousSpace<1> (q = 2,
 * include/continuous_space.hpp:33-152), DiscontinuousSpace<0> (q = 1). */
enum { HBEM_SPACE_P0 = 1, HBEM_SPACE_P1 = 2 };

typedef struct hbem_builder_s* hbem_builder;
typedef struct hbem_solop_s* hbem_solop;

int hbem_version(void);
const char* hbem_status_string(int status);
/* last error message of the calling thread (static storage) */
const char* hbem_last_error(void);
/* select the CUDA device used by handles created afterwards */
int hbem_set_device(int device);
/* Process-wide switches, for tests and measurements:
 *   "lu_cluster_panels" (default 1): LU panels taller than one CTA's shared memory
 *   are factored by a thread-block cluster holding the panel in distributed shared
 *   memory; 0 factors them in global memory.
 *   "lu_tensor_cores" (default 1): the complex-FP32 LU of the mixed-precision randomized
 *   SVD does its trailing updates on the tensor cores (3xTF32); 0 uses FP32 FMA.
 *   "svd_fast" (default 1): dense sigma_min / sigma' / sigma'' (direct::sv*) of matrices
 *   up to order 100 by FP32 Jacobi plus FP64 refinement of the near singular triplets
 *   (one FP64 LU per matrix); 0 always uses the FP64-polished Jacobi kernel.
 *   Matrices the fast kernel cannot finish are redone by the polished kernel; that
 *   fallback is per call and per host thread and leaves this switch unchanged.
 *   "svd_fast_force_redo" (default 0): 1 sends every fast-kernel result through that
 *   fallback as well (more work, same results), so tests can exercise it.
 *   "svd_pair_max" (default 16, >= 0): launches of the fast kernel with at most this
 *   many matrices run each matrix on a cluster of two CTAs (FP32 Jacobi beside the
 *   FP64 LU, inverse iterations split by columns): lower latency per matrix, results
 *   bit-identical to the one-CTA form; 0 never pairs.
 *   "arnoldi_maxit" (default 1000, >= 1): iteration cap of hbem_arnoldi_sv_batch*.
 *   "mlp_tensor_cores" (default 1): the MLP's BF16 products on tcgen05; 0 uses FP32 FMA.
 *   "singular_table" (default 1): coincident / adjacent panel pairs read the
 *   k-independent data of their composite quadrature points (distance, tangent and
 *   normal products, weights) from a table the builder makes once (up to 256 MB);
 *   0 computes it in the kernel for every wavenumber and medium.
 *   "singular_split" (default 1): assembly launches of few wavenumbers (coincident /
 *   adjacent pairs x media below four CTAs per SM) split every such pair over several
 *   CTAs of equal work and add the parts in a second launch: lower latency for one
 *   T(k); sums in another order (results agree to ~1e-15).  The pipelined plain search
 *   does not split (its launches share the GPU).
 *   "plain_speculate" (default 1): speculative bisection points in the plain
 *   search's small Newton rounds (hbem_find_resonances_plain).
 *   "autotune" (default 0): the panel-pair assembly times each layout of its general
 *   pairs (a thread per pair, or a warp per pair with 1-16 pairs per warp) on the
 *   first launch of every (panels, order, jobs rounded up to a power of two,
 *   derivative order, real k, panel kind) and uses the fastest from then on; the
 *   choices persist in the file the environment variable HBEM_TUNE_CACHE names, if
 *   any.  Results of different layouts agree to rounding (~1e-15).
 *   "plain_async" (default 1): the plain search (with warm starts) as one pipeline of
 *   streams: grid chunks overlapping, each candidate's bracket ends and Newton points
 *   as soon as their inputs are known, instead of one batch per phase and lock-step
 *   Newton rounds; the same Newton steps either way.
 *   "plain_spec_async" (default 2), "plain_spec_deep" (default 2): with "plain_async",
 *   a candidate speculates bisection points while at most plain_spec_async candidates
 *   are unfinished, two bisection levels deep while at most plain_spec_deep are.
 *   "plain_warm_start" (default 1): in the plain search, the dense kernel's FP32
 *   Jacobi at a bracket end or Newton point starts from the right singular vectors
 *   of the nearest wavenumber already evaluated (same stopping rule, fewer sweeps). */
int hbem_set_option(const char* name, int value);
/* the current value of one of the switches above */
int hbem_get_option(const char* name, int* value);

/* Instrumentation (no counterpart in the reference, which prints std::chrono
 * timings, gen_sol_op.cpp:89-99 and randsvd.cpp:27-47): kernel launches issued
 * by this library, and -- when timing is enabled -- CUDA-event time, launch count
 * and processed (quadrature point x medium) count of the panel-pair assembly
 * launches, timed on the stream they run on.                 */
void hbem_stats_enable_timing(int enable);
void hbem_stats_reset(void);
void hbem_stats_read(long long* launches, double* assembly_ms, long long* assembly_launches,
                     long long* assembly_points);
/* The timed assembly's (point x medium) count split9[9] by kind and derivative
 * order d: [d] general pairs, [3 + d] singular pairs reading their k-independent
 * point data from the builder's table, [6 + d] singular pairs computing it.      */
void hbem_stats_read_points(long long* split9);

/* H0^(1), H1^(1) of n arguments on the device: complex_bessel::Hankel1Real01::h1_01
 * for real x (include/cbessel.hpp:236-288) when complex_arg == 0 (z_host holds n
 * reals), HankelH1(0|1, z) / H1_01 (include/cbessel.hpp:156, 300) otherwise (n
 * interleaved complex).  h0_host, h1_host: n interleaved complex each.            */
int hbem_hankel01(int n, const double* z_host, int complex_arg, double* h0_host, double* h1_host);

/* ------------------------------------------------------------------ builder */

/* BuilderData(mesh, test_space, trial_space, order) + GalerkinBuilder(data)
 * (include/galerkin_builder.hpp:43-46, 200; source/galerkin_builder.cpp:17-187).
 * The mesh is given as panels; q_test, q_trial select ContinuousSpace<1>
 * (HBEM_SPACE_P1, include/continuous_space.hpp:33-152) or DiscontinuousSpace<0>
 * (HBEM_SPACE_P0, include/discontinuous_space.hpp:33-127) for the test and trial
 * spaces.  As in the reference, the double layer is test x trial, the hypersingular
 * trial x trial and the single layer test x test (galerkin_builder.cpp:936-946);
 * with test != trial spaces the double layer takes every ordered panel pair
 * (the non-square branch, galerkin_builder.cpp:966-1009).                         */
int hbem_builder_create(int npanels, const int* kinds, const double* params, int order, int q_test, int q_trial,
                        hbem_builder* out);
int hbem_builder_destroy(hbem_builder b);
/* dimensions: panels, test/trial space dimension, quadrature order, all-lines flag */
int hbem_builder_info(hbem_builder b, int* npanels, int* dim_test, int* dim_trial, int* order, int* lines);
/* BuilderData::is_adjacent (source/galerkin_builder.cpp:189-201) */
int hbem_builder_is_adjacent(hbem_builder b, int i, int j, int* adjacent, int* swap);

/* GalerkinBuilder::assembleDense(k, c, layers, d) for the full matrix
 * (include/galerkin_builder.hpp:221-222; source/galerkin_builder.cpp:918-1018).
 * Errors as the reference: c < 1, Im k < 0 or d > 2 -> HBEM_ERR_INVALID.       */
int hbem_assemble_dense(hbem_builder b, double k_re, double k_im, double c, unsigned layers, unsigned d);
/* assembleDense(k, c, layers, d, row, col, rows, cols) with the reference's sub-matrix
 * rule (galerkin_builder.cpp:918-1009): only panel pairs with one panel in
 * [row, row + rows) and the other in [col, col + cols) contribute, to the dof block
 * [row, row + rows) x [col, col + cols); rows, cols = 0 mean N.  Every layer is
 * rows x cols (the reference sizes V rows x rows and W cols x cols).  hbem_get_layer*
 * then return rows x cols matrices.                                               */
int hbem_assemble_dense_sub(hbem_builder b, double k_re, double k_im, double c, unsigned layers, unsigned d,
                            unsigned row, unsigned col, unsigned rows, unsigned cols);
/* getDoubleLayer / getHypersingular / getSingleLayer(d) (include/galerkin_builder.hpp:262-276):
 * copies the N x N complex matrix to host_out; HBEM_ERR_INVALID if the layer or
 * derivative was not assembled by the last hbem_assemble_dense.                  */
int hbem_get_layer(hbem_builder b, unsigned layer, unsigned d, double* host_out);
/* same, device pointer owned by the builder, valid until the next assembly */
int hbem_get_layer_device(hbem_builder b, unsigned layer, unsigned d, const void** dev_ptr);

/* ------------------------------------------------------------------ solutions operator */

/* SolutionsOperator(builder_data, proj) (include/gen_sol_op.hpp:40-60;
 * source/utilities/gen_sol_op.cpp:23-43): mass matrix of the builder's test and
 * trial spaces and projection factor.  proj != 0 needs test space = trial space:
 * for P0 x P1 the mass matrix is not symmetric and the reference's LDL^T would read
 * only its lower triangle (HBEM_ERR_UNSUPPORTED here).  The transmission problem
 * (hbem_tp_*) needs P1/P1.                                                      */
int hbem_solop_create(hbem_builder b, int proj, hbem_solop* out);
int hbem_solop_destroy(hbem_solop s);
/* SolutionsOperator::mass_matrix() (include/gen_sol_op.hpp:105): N x N real, column-major */
int hbem_mass_matrix(hbem_solop s, double* host_out);
/* gen_sol_op / gen_sol_op_1st_der / gen_sol_op_2nd_der (source/utilities/gen_sol_op.cpp:50-196):
 * T and, for d >= 1, its k-derivatives, each 2N x 2N, written consecutively to
 * T_host ((d + 1) matrices).  The derivative matrices are the projected
 * derivative blocks (the reference writes them all into T, gen_sol_op.cpp:151,194). */
int hbem_gen_sol_op(hbem_solop s, double k_re, double k_im, double c_o, double c_i, unsigned d, double* T_host);
/* batched form over nk real wavenumbers; T_dev receives [nk][d + 1][2N][2N] */
int hbem_gen_sol_op_batch_device(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d,
                                 void* T_dev);
/* Many scatterers at once (the batching path of the reference's drivers, which loop
 * over scatterers and sweep k with std::execution::par,
 * examples/roots_newton_polygon_rsvd.cpp:172-177): operator i at counts[i] real
 * wavenumbers k_host[sum_{j<i} counts[j] + q] with inner index c_i_host[i]; T(k) and
 * its first d derivatives of operator i into T_dev[i] (layout of
 * hbem_gen_sol_op_batch_device).  The panel-pair quadrature of every (scatterer, k,
 * medium) runs in one general-pair and one singular-pair launch per panel kind
 * (lines / arcs), whatever the panel counts; the work is issued on the first
 * operator's stream and finished on return.                                       */
int hbem_gen_sol_op_multi_device(const hbem_solop* ops, int nops, const int* counts, const double* k_host,
                                 const double* c_i_host, double c_o, unsigned d, void* const* T_dev);

/* ------------------------------------------------------------------ scatterers (host only) */

/* scatterer::read (include/scatterer.hpp:39; source/utilities/scatterer.cpp:30-82): one
 * vertex "x,y" per line, whitespace anywhere ignored, empty lines skipped; every
 * field must parse as a double (a '#' line is rejected, as the reference's parser
 * does); the widest row must have two fields (a shorter row is padded with zeros).
 * Coordinates are multiplied by scale.  With x_host or y_host NULL only *nvert is
 * returned.  HBEM_ERR_INVALID on an unreadable or malformed file or cap < nvert.  */
int hbem_scatterer_read(const char* fname, double scale, double* x_host, double* y_host, int cap, int* nvert);
/* scatterer::length (scatterer.cpp:84-93): perimeter of the closed polygon */
double hbem_polygon_length(const double* x, const double* y, int n);
/* scatterer::auto_num_panels (scatterer.cpp:95-112): round(perimeter / (f shortest side)) */
unsigned hbem_auto_num_panels(const double* x, const double* y, int n, double f);
/* scatterer::make_N_polygonal_panels (scatterer.cpp:114-155): exactly N line panels,
 * evenly split per edge, counts proportional to the edge lengths.  params: 5 doubles
 * per panel (x1 y1 x2 y2 0, kind HBEM_PANEL_LINE); with params NULL only *npanels is
 * returned.                                                                       */
int hbem_polygon_panels(const double* x, const double* y, int n, unsigned N, double* params, int cap,
                        int* npanels);
/* scatterer::make_polygonal_panels (scatterer.cpp:157-277): about N line panels graded
 * geometrically towards the corners (the first panel at a corner is rf + (1 - rf)(1 -
 * cos angle)/2 times the uniform length); edges with fewer than three panels, or
 * refinement_factor >= 1, are split evenly.                                        */
int hbem_polygon_panels_graded(const double* x, const double* y, int n, unsigned N, double refinement_factor,
                               double* params, int cap, int* npanels);
/* Panel count of examples/find_resonances.cpp:111-124: Brent's minimiser on
 * [N0, N0 / rfac], N0 = degf L k_max / (2 pi), of |2 pi / (degf k_max) - longest panel
 * of make_polygonal_panels(round N, rfac)|; *npanels = round of the minimiser.       */
int hbem_choose_num_panels(const double* x, const double* y, int n, double k_max, double degf, double rfac,
                           unsigned* npanels);

/* ------------------------------------------------------------------ transmission problem and fields */

/* Incoming waves: records of 7 doubles {type, amplitude, x0, y0, angle, eps, order}
 * (incoming::wavespec_t, include/incoming.hpp:28-43); type 0 Plane, 1 CircularJ,
 * 2 CircularY, 3 FourierHankel1, 4 FourierHankel2, 5 Herglotz.  Circular and
 * Fourier-Hankel records need a real wavenumber (HBEM_ERR_UNSUPPORTED otherwise). */
enum { HBEM_WAVE_PLANE = 0, HBEM_WAVE_CIRCULAR_J = 1, HBEM_WAVE_CIRCULAR_Y = 2, HBEM_WAVE_FOURIER_HANKEL1 = 3,
       HBEM_WAVE_FOURIER_HANKEL2 = 4, HBEM_WAVE_HERGLOTZ = 5 };
/* incoming::load (source/utilities/incoming.cpp:48-92): one record per line,
 * "Type, amplitude, x0, y0, angle[, eps]" or "Type, amplitude, x0, y0, order";
 * whitespace ignored, empty and '#' lines skipped.  With waves NULL only *nwaves is
 * returned.  HBEM_ERR_INVALID where the reference returns false.                */
int hbem_incoming_load(const char* fname, double* waves, int cap, int* nwaves);
/* incoming::compute / compute_del (incoming.cpp:95-147) at npts points xy (x, y
 * pairs): u_host npts complex, du_host (may be NULL) npts x (du/dx, du/dy).      */
int hbem_incoming_eval(const double* waves, int nwaves, double k_re, double k_im, const double* xy_host, int npts,
                       double* u_host, double* du_host);
/* tp::direct_second_kind::solve (include/solvers.hpp:101-107, solvers.cpp:116-164)
 * on the mesh of s, which must be created with proj = 0 (the reference builds an
 * unprojected SolutionsOperator): T(k) x = [-K_o + M/2, V_o; W_o, K_o^T + M/2] (u_inc,
 * du_inc/dn at the panel start points).  traces_host: 2N complex (Dirichlet, then
 * Neumann coefficients).  HBEM_ERR_NONFINITE / HBEM_ERR_SINGULAR with the
 * reference's messages.                                                          */
int hbem_tp_solve(hbem_solop s, const double* waves, int nwaves, double k_re, double k_im, double c_o, double c_i,
                  double* traces_host);
/* tp::direct_second_kind::solve_in_rectangle (include/solvers.hpp:137-200,
 * solvers.cpp:165-391): the scattered (total_field = 0) or total field on the
 * nx x ny grid of [ll, ur] (x index fastest, column-major like Eigen::ArrayXXcd),
 * by the Green representation with order_green Gauss points per panel over the
 * traces splined along arc length; grid points on the boundary take the Dirichlet
 * trace, panels closer than 1e-2 / |kappa| are integrated by a graded composite rule.
 * traces_host: the 2N traces of hbem_tp_solve, or NULL to solve first (then s must
 * be unprojected).  grid_x_host, grid_y_host (may be NULL): the grid coordinates.  */
int hbem_tp_field_grid(hbem_solop s, const double* waves, int nwaves, double k_re, double k_im, double c_o,
                       double c_i, unsigned order_green, double ll_x, double ll_y, double ur_x, double ur_y, int nx,
                       int ny, int total_field, const double* traces_host, double* field_host, double* grid_x_host,
                       double* grid_y_host);
/* Instrumentation of the last hbem_tp_field_grid call of this thread: CUDA-event time
 * of the grid kernel, (grid point, boundary node) pairs it summed, near pairs.     */
void hbem_field_stats(double* grid_kernel_ms, long long* point_node_pairs, long long* near_pairs);

/* Local minima of sigma_min from candidate brackets [a_i, b_i] (the confirmation step
 * of the learned proposal; the Newton phase of hbem_find_resonances_plain): brackets
 * with sigma'(a) < 0 < sigma'(b) go to safeguarded Newton on sigma' (rtsafe, from the
 * secant zero of sigma'); brackets whose ends both rise or both fall are moved one
 * width left or right, at most max_shift times.  Roots ascending, merged within tol;
 * *n_evals counts the sigma evaluations.                                           */
int hbem_refine_brackets(hbem_solop s, const double* a_host, const double* b_host, int ncand, double c_o, double c_i,
                         double tol, int max_shift, double* roots_host, int max_roots, int* nroots, int* n_evals);

/* Many scatterers at once (no counterpart in the reference, whose drivers loop over
 * scatterers): hbem_sweep_sigma for operator i at counts[i] consecutive wavenumbers of
 * k_host with inner index c_i_host[i]; each operator's T(k) batch and dense SVD are
 * enqueued on its own stream before any is awaited.  out_host: 3 values per point. */
int hbem_sweep_sigma_multi(const hbem_solop* ops, int nops, const int* counts, const double* k_host,
                           const double* c_i_host, double c_o, unsigned d, double* out_host);
/* hbem_find_resonances_plain and hbem_refine_brackets for nops (operator, window)
 * pairs in lock step: every phase is one hbem_sweep_sigma_multi call.  Roots are
 * concatenated in operator order, root_counts[i] of them for operator i; brackets of
 * operator i are the counts[i] consecutive entries of a_host, b_host.             */
int hbem_find_resonances_plain_multi(const hbem_solop* ops, int nops, const double* k_min, const double* k_max,
                                     int npoints, double c_o, const double* c_i, double tol, double* roots_host,
                                     int max_roots, int* root_counts, int* n_evals);
int hbem_refine_brackets_multi(const hbem_solop* ops, int nops, const int* counts, const double* a_host,
                               const double* b_host, double c_o, const double* c_i, double tol, int max_shift,
                               double* roots_host, int max_roots, int* root_counts, int* n_evals);

/* ------------------------------------------------------------------ learned proposal network */

/* The multilayer perceptron of the learned resonance proposal (no counterpart in the
 * reference): n_in -> width (GELU) x depth -> n_out, BF16 products with FP32
 * accumulation on the tensor cores, FP32 master weights and Adam.  Parameters and
 * gradients as one FP32 vector: per layer W (out x in, row-major) then b.         */
typedef struct hbem_mlp_s* hbem_mlp;
int hbem_mlp_create(int n_in, int width, int depth, int n_out, unsigned long long seed, hbem_mlp* out);
int hbem_mlp_destroy(hbem_mlp m);
int hbem_mlp_num_params(hbem_mlp m, long long* count);
int hbem_mlp_get_params(hbem_mlp m, float* host);
int hbem_mlp_set_params(hbem_mlp m, const float* host);
/* Y (batch x n_out) from X (batch x n_in), row-major host arrays */
int hbem_mlp_forward(hbem_mlp m, const float* X_host, int batch, float* Y_host);
/* mean squared error against T (batch x n_out) and, when grads_host is not NULL, its
 * gradient with respect to the parameters */
int hbem_mlp_gradients(hbem_mlp m, const float* X_host, const float* T_host, int batch, float* loss_host,
                       float* grads_host);
/* one Adam step (beta 0.9 / 0.999, eps 1e-8) on that loss */
int hbem_mlp_train_step(hbem_mlp m, const float* X_host, const float* T_host, int batch, float lr, float* loss_host);
/* C (FP32, M x N, row-major, ldc) = A (BF16, M x K, lda) B (BF16, N x K, ldb)^T on the
 * device: the network's product kernel; M, N multiples of 128, K of 64.            */
int hbem_bf16_gemm_device(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, void* C,
                          long long ldc, int tensor_cores);

/* ------------------------------------------------------------------ singular values */

/* direct::sv / sv_1st_der / sv_2nd_der for the smallest singular value
 * (include/singular_values.hpp; source/utilities/singular_values.cpp:7-147), batched:
 * matrices T_dev + m*mat_stride (+ der_stride for T', + 2*der_stride for T''),
 * strides in complex elements.  out_host[3m + t] = sigma, sigma', sigma'' (d >= t).
 * sig_all_host, when not NULL, receives all n singular values of each matrix.     */
int hbem_sv_dense_batch_device(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                               long long der_stride, double* out_host, double* sig_all_host);

/* Allocation-free form of hbem_sv_dense_batch_device.  No counterpart in the
 * reference.  For callers that must not allocate device memory -- code running
 * while a memory pool or allocator is locked, inside another library's
 * pre-planned memory budget, or on a stream whose work must not trigger
 * cudaMalloc / cudaFree synchronisation -- this call allocates nothing: it
 * launches on `stream` (a cudaStream_t, NULL for the default stream) and returns
 * without waiting.  The caller passes the inputs and the outputs on the device:
 * out_dev (nmat x 3 doubles: sigma, sigma', sigma'') and status_dev (nmat ints,
 * 0 = converged, 4 = Jacobi sweep limit reached).
 * Working memory is a fixed 8 MiB array inside the library's device image
 * (held on every GPU that loads the library until the process exits).  Limits:
 * n <= 116 and nmat * n * n <= 524288; larger requests return HBEM_ERR_INVALID.
 * T_dev, out_dev and status_dev must be device (or managed) memory of the current
 * device; other pointers return HBEM_ERR_INVALID.
 * The first call on each device resolves the array's device address (with that
 * device current); make that first call before any stream capture.  Under lazy
 * module loading (CUDA_MODULE_LOADING=LAZY, the CUDA 12+ default) that first call
 * also loads the library's dense-SVD module with its array, which allocates and
 * synchronises once: make it during set-up, outside the section that must not
 * allocate.  After a device reset (cudaDeviceReset) the array is gone; the next
 * call notices that and resolves it again, with the same one-time cost.  All calls
 * share the array and it keeps the previous call's contents: calls whose work
 * overlaps on the GPU (different streams, or concurrent host threads) race on it. */
int hbem_sv_dense_batch_noalloc(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                                long long der_stride, double* out_dev, int* status_dev, void* stream);

/* same with host matrices (copied to the device): T_host holds nmat blocks of
 * (d + 1) consecutive n x n matrices (T, T', T'') */
int hbem_sv_dense_batch(int n, int nmat, unsigned d, const double* T_host, double* out_host, double* sig_all_host);

/* randomized_svd::randGaussian(nr, nc) (include/randsvd.hpp:23-30): (U[0,1] + i U[0,1])/sqrt2
 * entries, column-major nr x nc, from a seeded generator (the reference seeds from
 * std::random_device, so its sketches are not reproducible).                     */
int hbem_rand_sketch(int nr, int nc, unsigned long long seed, double* R_host);

/* randomized_svd::sv (d = 0), sv_der (d = 1) and sv_der2 (d = 2)
 * (include/randsvd.hpp:53,64,77; source/utilities/randsvd.cpp:99-216) for a batch
 * of nmat matrices of order n: LU of T, q subspace iterations with the n x s sketch
 * R (s <= 32), sigma ~ 1/sigma_max(T^-H Q).  sigma' = Re u^H T' v from the Ritz
 * vectors of the sketch; sigma'' by the reference's bordered 2n x 2n system (column
 * m of W - sigma I replaced by -u).  Matrices whose LU and sketch fit in shared
 * memory (n <= 108 at s = 16) run in one kernel per matrix, larger ones through the
 * batched global-memory LU below.  out_host[(d+1) m + t] = sigma, sigma', sigma''.
 * T_host: nmat blocks of d + 1 matrices (T, T', T'').  HBEM_ERR_SINGULAR if an LU of
 * T meets a zero pivot; a singular bordered system gives sigma'' = NaN, as the
 * reference's unguarded solve would.                                             */
int hbem_rsvd_sv_batch(int n, int nmat, unsigned d, const double* T_host, const double* R_host, int s, int q,
                       double* out_host);
int hbem_rsvd_sv_batch_device(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                              long long der_stride, const void* R_dev, int s, int q, double* out_host);
/* The same with a precision choice for the global-memory path: precision 0 = FP64
 * LU and solves; 1 = complex-FP32 LU (FP32 trailing updates), FP32 solves in the
 * subspace iterations, and `refine` passes (>= 1; 1 = none) of FP64-residual
 * iterative refinement for the final T^-H Q and the Ritz-vector solves.  Matrices
 * on the shared-memory path are computed in FP64 whatever the choice.            */
int hbem_rsvd_sv_batch_device_ex(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                                 long long der_stride, const void* R_dev, int s, int q, int precision, int refine,
                                 double* out_host);

/* arnoldi::sv (d = 0), sv_1st_der (d = 1) and sv_2nd_der (d = 2)
 * (include/singular_values_arnoldi.hpp:29-66; source/utilities/singular_values_arnoldi.cpp:19-246)
 * for a batch of nmat matrices of order n: the `count` smallest singular values in
 * ascending order, each with its k-derivatives.  The reference runs ARPACK on
 * [0 T^-H; T^-1 0] through one LU of T; here a block subspace iteration on
 * T^-1 T^-H (32 columns at most, seeded start block) with a Rayleigh-Ritz step per
 * iteration stops when every wanted Ritz pair of that operator has residual
 * <= acc |theta| (ARPACK's test; acc <= 0 means machine precision, and acc is
 * raised to 64 eps, the FP64 floor of the iteration).  out_host[(d+1)(m count + j) + t]
 * = sigma_j, sigma_j', sigma_j'' (t <= d).  sigma' = Re u^H T' v of the Ritz triplet;
 * sigma'' by the reference's bordered 2n x 2n system.  count up to 28 (or up to n
 * when n <= 32) runs the block iteration; larger counts with d = 0 take all n
 * singular values from the dense Jacobi kernel, larger counts with d > 0 give
 * HBEM_ERR_UNSUPPORTED.  status_host / iters_host (may be NULL): per matrix 0
 * converged, 5 zero pivot in the LU of T (results NaN), 6 iteration cap reached
 * (set_option "arnoldi_maxit", default 1000; results are the last iterate's) and the
 * number of block iterations.  Returns HBEM_ERR_SINGULAR / HBEM_ERR_NOCONV when any
 * matrix has status 5 / 6, with out_host filled either way.  T_host: nmat blocks
 * of d + 1 matrices (T, T', T'').                                                */
int hbem_arnoldi_sv_batch(int n, int nmat, unsigned d, int count, double acc, const double* T_host,
                          double* out_host, int* status_host);
int hbem_arnoldi_sv_batch_device(int n, int nmat, unsigned d, int count, double acc, const void* T_dev,
                                 long long mat_stride, long long der_stride, double* out_host, int* status_host,
                                 int* iters_host);

/* Batched complex64 update C_m -= A_m B_m (column-major, leading dimensions lda, ldb,
 * ldc, batch strides sa, sb, sc in elements): the trailing update of the LU's
 * complex-FP32 factorisation (the FP32 stand-in for the trailing GEMMs of Eigen's
 * PartialPivLU at source/utilities/randsvd.cpp:104).  tensor_cores = 1: tcgen05
 * MMAs with 3xTF32 split products and FP32 accumulation, K in chunks of 32 into one
 * tensor-memory accumulator; 0: FP32 FMA.                                        */
int hbem_cgemm_f32_batch_device(int m, int n, int k, const void* A, long long lda, long long sa, const void* B,
                                long long ldb, long long sb, void* C, long long ldc, long long sc, int nmat,
                                int tensor_cores);

/* Batched LU with partial pivoting, in place (Eigen::PartialPivLU<MatrixXcd> at
 * source/utilities/randsvd.cpp:104,205): nmat column-major complex128 matrices of
 * order n at A_dev + m * stride (elements).  piv_dev[m n + k] = row exchanged with
 * row k at step k (0-based LAPACK ipiv).  info_host (may be NULL): per matrix 0 or
 * 1 + the first step with a zero pivot; any zero pivot -> HBEM_ERR_SINGULAR.     */
int hbem_lu_factor_batch_device(int n, int nmat, void* A_dev, long long stride, int* piv_dev, int* info_host);
/* The same in complex FP32 (the factorisation behind the mixed-precision randomized
 * SVD): complex64 matrices; from order 256 on in 128-column blocks whose trailing
 * updates run on the tensor cores with 3xTF32 products and FP32 accumulation
 * (set_option "lu_tensor_cores" 0: FP32 FMA and 32-column panels).  HBEM_ERR_NOCONV
 * if a tensor-core completion wait timed out.                                   */
int hbem_lu_factor_batch_device_f32(int n, int nmat, void* A_dev, long long stride, int* piv_dev, int* info_host);
/* Solve with the factors (PartialPivLU::solve, and .adjoint().solve for trans = 1):
 * X_m <- T_m^-1 X_m or T_m^-H X_m, nrhs columns at X_dev + m * xstride, leading
 * dimension n.                                                                   */
int hbem_lu_solve_batch_device(int n, int nmat, int trans, const void* LU_dev, long long stride, const int* piv_dev,
                               int nrhs, void* X_dev, long long xstride);

/* Number of panels N of the operator's mesh (T is 2N x 2N).                       */
int hbem_solop_info(hbem_solop s, int* npanels);

/* sigma_min(k) along a list of real wavenumbers by randomized_svd::sv on a seeded
 * sketch of width `sketch` with q subspace steps (the sampling evaluator of
 * examples/find_resonances.cpp:135-139); precision as hbem_rsvd_sv_batch_device_ex. */
int hbem_sigma_rsvd_sweep(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, int sketch, int q,
                          int precision, unsigned long long seed, double* sigma_out);

/* sigma_min(k) and its derivatives along a list of real wavenumbers, end to end:
 * gen_sol_op_*der + direct::sv_*der per k (examples/roots_newton_circle.cpp:111-138).
 * out_host[3i + t]. */
int hbem_sweep_sigma(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d, double* out_host);

/* Plain resonance search on [k_min, k_max] with npoints grid points
 * (examples/roots_newton_polygon_rsvd.cpp:172-265 with the dense sigma of
 * examples/roots_newton_circle.cpp): sigma on the grid; 3-point local minima;
 * sigma' at both bracket ends, validation sigma'(left) < 0 < sigma'(right); quartic
 * Hermite model minimised by Brent; rtsafe on sigma' with sigma'' to tolerance tol.
 * Where the one-CTA dense kernel takes the order, the search runs as one pipeline
 * on several streams (option "plain_async", default 1): the grid in chunks whose
 * dense sigma overlaps the next chunk's assembly, each candidate's bracket ends as
 * soon as the grid around it is known, and its Newton points one after another,
 * independently of the other candidates; otherwise each phase is one batch, the
 * Newton steps of all candidates in one batch per round.  The values are the same,
 * except that in the pipeline a Newton step of at most 1e-6 takes T, T', T'' from the
 * point just evaluated by their Taylor polynomials instead of assembling them (sigma'
 * there agrees with the assembled value to ~1e-11, the roots to ~1e-12).
 * roots_host receives up to max_roots roots, *nroots their count; grid_host
 * (npoints x 3, may be NULL) sigma at every grid point and sigma' at the bracket
 * ends (NaN where not evaluated); *n_evals the number of T(k) evaluated.
 * Where the one-CTA dense sigma kernel takes the order (2N <= 100), while few
 * candidates are left a candidate at its first point or just after a bisection step
 * also has the points a further bisection step of rtsafe could move to evaluated
 * (option "plain_speculate", default 1); when that step follows, its point needs no
 * evaluation of its own.  Every candidate takes the same steps as without
 * speculation, so the roots are the same; *n_evals counts the evaluations the
 * search used (unused speculative points excluded).                               */
int hbem_find_resonances_plain(hbem_solop s, double k_min, double k_max, int npoints, double c_o, double c_i,
                               double tol, double* roots_host, int max_roots, int* nroots, double* grid_host,
                               int* n_evals);
/* The same search with every root checked (no counterpart in the reference, whose
 * drivers report rtsafe's result as is): check_host[2i], check_host[2i + 1] receive
 * sigma' at roots_host[i] - tol and roots_host[i] + tol, so that a root is verified
 * when check_host[2i] <= 0 <= check_host[2i + 1].  With the Newton candidates on
 * their own streams (option "plain_async") a candidate's two points are evaluated as
 * soon as it converges, beside the other candidates' iterations, with T and T' there
 * taken from the last Newton point's T, T', T'' by their Taylor polynomials (the
 * points lie within 2 tol of it, so the terms left out are below FP64 rounding;
 * no assembly); otherwise the points are assembled, in one batch after the search.  */
int hbem_find_resonances_plain_verified(hbem_solop s, double k_min, double k_max, int npoints, double c_o, double c_i,
                                        double tol, double* roots_host, int max_roots, int* nroots, double* grid_host,
                                        int* n_evals, double* check_host);

/* Adaptive resonance search (examples/find_resonances.cpp:128-250 with the sampler
 * opt_subdiv, source/utilities/find_roots.cpp:1615-1726): batches of batch_size
 * random wavenumbers (seeded; uniform, then normal about the error of a Steffen
 * monotone spline through the samples) with sigma_min by randomized_svd::sv on a
 * `sketch`-wide sketch with q steps, until the number of local minima has not grown
 * for `limit` batches (samples kept sample_tol (k_max - k_min) apart); each minimum
 * improved on a Floater-Hormann rational interpolant (order 5) and refined by Brent
 * minimisation of sigma_min (dense sigma for T up to order 100, else a 16-wide
 * sketch) to relative interval tol, all candidates in one batch per round.  The
 * mesh is the caller's (the reference's panel-count choice is left to it).
 * roots_host: up to max_roots minima, *nroots their count; *n_samples, *n_evals
 * (may be NULL) the sample count and the T(k) evaluations.                        */
int hbem_find_resonances_adaptive(hbem_solop s, double k_min, double k_max, double c_o, double c_i, int batch_size,
                                  int limit, double sample_tol, double tol, unsigned long long seed, int sketch,
                                  int q, double* roots_host, int max_roots, int* nroots, int* n_samples,
                                  int* n_evals);

/* ------------------------------------------------------------------ root finding (host) */

typedef double (*hbem_fn)(double x, void* user);
typedef void (*hbem_fn_both)(double x, double* f, double* df, void* user);
typedef void (*hbem_fn_batch)(const double* x, int n, double* y, void* user);

/* rtsafe (include/find_roots.hpp:37-49; source/utilities/find_roots.cpp:117-217):
 * safeguarded Newton; returns the root, sets *root_found and *num_iter. */
double hbem_rtsafe(hbem_fn f, hbem_fn_both f_both, void* user, double x1, double x2, double tol, int* root_found,
                   unsigned* num_iter);
/* zbrent (include/find_roots.hpp:51-67; source/utilities/find_roots.cpp:19-115) */
double hbem_zbrent(hbem_fn f, void* user, double x1, double x2, double tol, int* root_found, unsigned* num_iter);
/* BrentMinimizer(a, b, tol).local_min_rc(status, value) (include/find_roots.hpp:181-233),
 * reverse communication: create, then call step with *status = 0 first; while the
 * returned *status > 0 evaluate f at the returned point and pass the value back;
 * *status = 0 returns the estimated minimiser.                                   */
int hbem_brent_rc_create(double a, double b, double tol, void** handle);
double hbem_brent_rc_step(void* handle, int* status, double value);
int hbem_brent_rc_destroy(void* handle);
/* brent_guess (find_roots.hpp:256; find_roots.cpp:1233-1313) and brent_gsl /
 * brent_gsl_with_values (find_roots.hpp:262-265; find_roots.cpp:1426-1473: Brent's
 * minimiser as GSL documents it, relative interval tolerance tol, 100 iterations at
 * most); NaN when f(guess) is not below f(a) and f(b), where GSL refuses the bracket. */
double hbem_brent_guess(hbem_fn f, void* user, double a, double b, double guess, double fguess, double tol,
                        unsigned* num_iter);
double hbem_brent_gsl(hbem_fn f, void* user, double a, double b, double guess, double tol, unsigned* num_iter);
double hbem_brent_gsl_with_values(hbem_fn f, void* user, double a, double fa, double b, double fb, double guess,
                                  double fguess, double tol, unsigned* num_iter);
/* BrentMinimizer(a, b, tol).local_min_rc driven to completion
 * (include/find_roots.hpp:181-233; source/utilities/find_roots.cpp:1003-1184) */
double hbem_brent_min(hbem_fn f, void* user, double a, double b, double tol);

/* opt_subdiv (find_roots.cpp:1615-1726) for any batched function f: samples sorted
 * by x into x_out / y_out (up to max_points; *n_points their number) and the
 * indices of interior local minima into minima_out (*n_minima).  The reference
 * seeds from std::random_device; here `seed` (SplitMix64, Box-Muller normals).   */
int hbem_opt_subdiv(hbem_fn_batch f, void* user, double x_min, double x_max, int batch_size, int limit, double tol,
                    unsigned long long seed, double* x_out, double* y_out, int max_points, int* n_points,
                    int* minima_out, int max_minima, int* n_minima);

#ifdef __cplusplus
}
#endif

#endif /* HBEM_H */
