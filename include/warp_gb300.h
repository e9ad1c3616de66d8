/*
 * warp_gb300.h -- C ABI of libwarp_gb300.so, the sm_103a (GB300) implementation of Warp's
 * finite-element linear-solve path.
 *
 * Conventions
 *   - All array arguments are DEVICE pointers unless named *_host.  Sizes are element counts.
 *   - Every call is stream-ordered on `stream` (a cudaStream_t; 0 = legacy default stream) and
 *     never synchronises the host, except where a host output is documented.
 *   - Return value: 0 on success, a negative GbStatus on failure; gb_last_error() returns the
 *     message (per host thread).  No exception crosses the ABI.
 *   - The library allocates no device memory: callers pass workspaces sized by the matching
 *     *_workspace_bytes() query (the Krylov handle owns only its CUDA graphs).
 *   - Kernels report device-side conditions by OR-ing GB_DEV_* bits into a caller-provided int32
 *     status word; waits inside kernels are bounded.
 * Reference citations are paths inside the Warp source tree.
 */
#ifndef WARP_GB300_H
#define WARP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gb_stream_t; /* == cudaStream_t */

enum { GB_OK = 0, GB_ERR_INVALID = -1, GB_ERR_CUDA = -2, GB_ERR_UNSUPPORTED = -3, GB_ERR_CAPACITY = -4 };
enum { GB_F32 = 0, GB_F64 = 1, GB_BF16 = 2, GB_F16 = 3 };
enum { GB_DEV_WAIT_TIMEOUT = 1, GB_DEV_BREAKDOWN = 2, GB_DEV_NONFINITE = 4, GB_DEV_STAGNATION = 8 };
enum { GB_KRYLOV_CG = 0, GB_KRYLOV_BICGSTAB = 1 };

/* ---- library ------------------------------------------------------------------------------ */
const char* gb_last_error(void);
void gb_clear_error(void);
int gb_version(void);

/* Programmatic dependent launch of the solver-loop kernels: mode 0 off, 1 (default) eager launches only,
 * 2 eager launches and launches into a capturing stream.  No reference counterpart: a launch option of
 * this library; results are identical in every mode.  Returns nonzero for a mode outside 0..2. */
int gb_set_pdl(int mode);
int gb_get_pdl(void);
int gb_device_arch(void);

/* ---- prefix sums ---------------------------------------------------------------------------
 * Replaces wp_array_scan_int_device (warp/native/warp.h:449; warp/native/scan.cu). */
size_t gb_scan_i32_workspace_bytes(int64_t n);
int gb_scan_i32(const int* in, int* out, int64_t n, int inclusive, void* workspace, size_t workspace_bytes,
                gb_stream_t stream);

/* Allocation-free variant of gb_scan_i32 (no counterpart in the reference): for callers that cannot
 * allocate device memory at all (a host application whose own arena owns all device memory and that
 * lets no library call cudaMalloc).  Its scratch is a fixed ~256 KB device array inside the library,
 * held by every GPU that loads it and shared by all calls: n <= gb_scan_i32_noalloc_max_n() (2^28) or
 * GB_ERR_CAPACITY; calls that overlap on the GPU race on the array.  The first call in a CUDA context
 * looks the array's address up (make that call before any stream capture). */
int64_t gb_scan_i32_noalloc_max_n(void);
int gb_scan_i32_noalloc(const int* in, int* out, int64_t n, int inclusive, gb_stream_t stream);

/* ---- triplets -> BSR -------------------------------------------------------------------------
 * gb_bsr_matrix_from_triplets_device replaces wp_bsr_matrix_from_triplets_device
 * (warp/native/warp.h:583-602; warp/native/sparse.cu:1168-1325): same arguments and semantics
 * (invalid indices and, when scalar_zero_mask != 0, all-zero blocks are pruned; masked_topology
 * keeps only blocks present in bsr_offsets/bsr_columns; tpl_block_offsets = inclusive run ends,
 * tpl_block_indices = triplet ids in stable sorted order; bsr_nnz_host receives offsets[nrow]
 * asynchronously and bsr_nnz_event (a cudaEvent_t, optional) is recorded after that copy), plus
 * a caller workspace and the stream.
 * gb_bsr_accumulate_triplet_values replaces the _bsr_accumulate_triplet_values launch
 * (warp/_src/sparse.py:1073-1090, 1503-1515). */
size_t gb_bsr_from_triplets_workspace_bytes(int nnz, int nrow, int ncol);
int gb_bsr_matrix_from_triplets_device(int block_size, int scalar_size, int row_count, int col_count, int nnz,
                                       const int* tpl_nnz, const int* tpl_rows, const int* tpl_columns,
                                       const void* tpl_values, uint64_t scalar_zero_mask, int masked_topology,
                                       int* tpl_block_offsets, int* tpl_block_indices, int* bsr_offsets,
                                       const int* bsr_row_counts, int* bsr_columns, int* bsr_nnz_host,
                                       void* bsr_nnz_event, void* workspace, size_t workspace_bytes,
                                       gb_stream_t stream);
int gb_bsr_accumulate_triplet_values(int dtype, int block_size, int row_count, const int* bsr_offsets,
                                     const int* tpl_block_offsets, const int* tpl_block_indices,
                                     const void* tpl_values, void* bsr_values, int nnz_upper, gb_stream_t stream);

/* ---- SpMV --------------------------------------------------------------------------------------
 * Replaces bsr_mv (warp/_src/sparse.py:4792-4913; kernels bsr_mv_kernel :4627-4665,
 * bsr_mv_tiled_kernel :4668-4715, bsr_mv_transpose_kernel :4718-4747).
 * y_out = alpha * op(A) x + beta * y_in; y_in may equal y_out; x must not alias y_out.
 * val_dtype GB_F32 / GB_F64 / GB_BF16; vec_dtype GB_F32 / GB_F64; ncap = entries available in
 * columns/values.  rows_per_cta / lanes_per_row / cap_blocks <= 0 (cap_blocks < 0) select the
 * built-in tile heuristic. */
int gb_bsr_mv(int block_rows, int block_cols, int nrow, int ncol, int64_t nnz_upper, int64_t ncap, const int* offsets,
              const int* row_counts, const int* columns, const void* values, int val_dtype, const void* x,
              const void* y_in, void* y_out, int vec_dtype, double alpha, double beta, int transpose,
              int rows_per_cta, int lanes_per_row, int cap_blocks, int* status, gb_stream_t stream);
int gb_bsr_mv_default_shape(int block_rows, int block_cols, int val_dtype, int nrow, int64_t nnz, int* rows_per_cta,
                            int* lanes_per_row, int* cap_blocks);

/* ---- diagonal, small operators, reductions -----------------------------------------------------
 * gb_bsr_get_diag: bsr_get_diag (warp/_src/sparse.py:2871-2887).
 * gb_bsr_inverse_diagonal: preconditioner(A, "diag"/"diag_abs") (warp/_src/optim/linear.py:236-329).
 * gb_diag_mv / gb_dense_mv: aslinearoperator diag_mv / dense_mv (warp/_src/optim/linear.py:135-233,
 *   kernels :2250-2287).
 * gb_dots: TiledDot.compute (warp/_src/optim/linear.py:309-576), fp64 accumulation, deterministic.
 * gb_axpby: array_axpy (warp/_src/utils.py). */
int gb_bsr_get_diag(int dtype, int br, int bc, int nrow, const int* offsets, const int* row_counts,
                    const int* columns, const void* values, void* out, gb_stream_t stream);
int gb_bsr_inverse_diagonal(int dtype, int bdim, int nrow, const int* offsets, const int* row_counts,
                            const int* columns, const void* values, int use_abs, void* inv, gb_stream_t stream);
int gb_diag_mv(int dtype, int64_t n, const void* A, const void* x, const void* y, void* z, double alpha, double beta,
               gb_stream_t stream);
int gb_dense_mv(int dtype, int m, int n, const void* A, const void* x, const void* y, void* z, double alpha,
                double beta, gb_stream_t stream);
size_t gb_dots_workspace_bytes(void);
int gb_dots(int dtype, int64_t n, int ncols, const void* const* xs, const void* const* ys, double* out,
            void* workspace, gb_stream_t stream);
int gb_axpby(int dtype, int64_t n, double alpha, const void* x, double beta, const void* y, void* out,
             gb_stream_t stream);

/* ---- fused Krylov solvers (CG / BiCGSTAB with Jacobi or no preconditioner) ----------------------
 * Replace CG._run (warp/_src/optim/linear.py:934-1032), BiCGSTAB._run (:1466-1574), their update
 * kernels (:2332-2373, :2426-2493), TiledDot and the capturable loop (_run_capturable_loop /
 * _update_condition / capture_while, :2086-2179; warp/native/warp.h:777).
 * gb_krylov_launch modes: 0 whole solve (init + device-side while loop, one graph), 1 init,
 * 2 `chunk_iters` iterations, 3 one eager iteration, 4 eager init.  Inside a caller's stream
 * capture, mode 0 appends the conditional loop to that capture.
 * CG handles run their iterations as one persistent cooperative launch (three phases per iteration
 * separated by grid barriers) when the device holds the whole SpMV grid at once; modes 0, 2 and 3
 * then launch it for "until converged", `chunk_iters` and one iteration.  gb_krylov_set_persistent
 * switches this off (three kernels per iteration under a conditional graph node) or back on and
 * reports through active_out (may be null) whether the persistent launch will be used. */
size_t gb_krylov_workspace_bytes(int kind, int block_dim, int nrow, int64_t nnz, int val_dtype);
int gb_krylov_create(int kind, int block_dim, int nrow, int64_t nnz, int64_t ncap, int val_dtype, int rows_per_cta,
                     int lanes_per_row, int cap_blocks, void* workspace, size_t workspace_bytes, void** handle_out);
int gb_krylov_destroy(void* handle);
int gb_krylov_set_operands(void* handle, const int* offsets, const int* row_counts, const int* columns,
                           const void* values, const float* dinv, const float* b, float* x, int x_is_zero, double tol,
                           double atol, int maxiter, int left_precond, gb_stream_t stream);
int gb_krylov_launch(void* handle, int what, int chunk_iters, gb_stream_t stream);
int gb_krylov_scalars(void* handle, int** iter, double** rr, double** atol_sq, int** status);
int gb_krylov_read(void* handle, int* host_ints3, double* host_doubles3, gb_stream_t stream);
int gb_krylov_vectors(void* handle, float** r, float** p, float** Ap);
int gb_krylov_set_persistent(void* handle, int enable, int* active_out);

/* ---- FP64 refinement pieces (no reference counterpart: the reference solves in the matrix
 * scalar type only; these wrap the fp32 solver of CG._run in iterative refinement) ------------- */
size_t gb_residual_f64_workspace_bytes(int block_dim, int nrow, int64_t nnz, int val_dtype);
int gb_residual_f64(int block_dim, int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* row_counts,
                    const int* columns, const void* values, int val_dtype, const double* x, const float* b,
                    double* r64, float* r32, double* norms, void* workspace, size_t workspace_bytes, int* status,
                    gb_stream_t stream);
int gb_axpy_f64_f32(int64_t n, double* x, const float* d, double alpha, gb_stream_t stream);
/* same residual in double-float (two-fp32) arithmetic from the interleaved (hi, lo) split x2 of x */
int gb_residual_df(int block_dim, int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* row_counts,
                   const int* columns, const void* values, int val_dtype, const void* x2, const float* b, double* r64,
                   float* r32, double* norms, void* workspace, size_t workspace_bytes, int* status,
                   gb_stream_t stream);
/* x += alpha * d (d may be null) and refresh the (hi, lo) split x2 (may be null) */
int gb_update_solution(int64_t n, double* x, void* x2, const float* d, double alpha, gb_stream_t stream);

/* ---- SpGEMM (bsr_mm) on the triplet assembly ----------------------------------------------------
 * Replace the bsr_mm pipeline (warp/_src/sparse.py:4200-4624, kernels :3620-3917): per block of x
 * count the product terms, emit (row, col, (x block, y block)) triplets (plus z's blocks when
 * beta != 0), assemble with gb_bsr_matrix_from_triplets_device, then sum each run. */
int gb_spgemm_count(int x_nrow, const int* x_offsets, const int* x_columns, const int* y_offsets, int x_nnz_cap,
                    int* count, gb_stream_t stream);
int gb_spgemm_emit(int x_nrow, const int* x_offsets, const int* x_columns, const int* y_offsets, const int* y_columns,
                   int x_nnz_cap, const int* start, int z_nrow, const int* z_offsets, const int* z_columns,
                   int z_nnz_cap, int z_base, int* rows, int* cols, void* pairs, gb_stream_t stream);
int gb_spgemm_values(int dtype, int nrow, const int* out_offsets, const int* run_ends, const int* run_ids,
                     const void* pairs, int br, int bk, int bc, const void* X, const void* Y, const void* Z,
                     double alpha, double beta, void* out, int nnz_upper, gb_stream_t stream);

/* ---- Q1 FEM assembly on regular grids ------------------------------------------------------------
 * gb_q1_assemble_triplets replaces fem.integrate's bilinear dispatch path for Q1 Grid2D/Grid3D
 * spaces (warp/_src/fem/integrate.py:1627-1878; warp/_src/fem/field/virtual.py:884-1116), writing
 * triplets in the reference's order.  gb_q1_assemble_rhs: the linear form sum_e M_e f
 * (integrate.py:1404-1625).  gb_grid_boundary_mask + gb_dirichlet_project: the nodal boundary
 * projector and project_linear_system (warp/_src/fem/dirichlet.py:69-124). */
int64_t gb_q1_triplet_count(int dim, int nx, int ny, int nz);
int gb_q1_assemble_triplets(int dim, int nx, int ny, int nz, int ncomp, const float* K0, const float* K1,
                            const float* coef0, float coef0_const, const float* coef1, float coef1_const, int* rows,
                            int* cols, float* vals, gb_stream_t stream);
/* Direct compact-BSR assembly of the same bilinear form (no counterpart entry point in the reference: it
 * produces the matrix that bsr_set_from_triplets builds from the triplets above, bit for bit -- same
 * pruning of all-zero triplets, same per-block summation order -- without writing or sorting them;
 * warp/_src/fem/integrate.py:1627-1878 + warp/native/sparse.cu:1168-1325).  K0/K1 are fp32 tables;
 * columns/values need gb_q1_bsr_nnz_max() blocks of capacity; bsr_nnz_host (optional) receives
 * offsets[nodes] asynchronously. */
int64_t gb_q1_bsr_nnz_max(int dim, int nx, int ny, int nz);
size_t gb_q1_assemble_bsr_workspace_bytes(int dim, int nx, int ny, int nz);
int gb_q1_assemble_bsr(int dim, int nx, int ny, int nz, int ncomp, const float* K0, const float* K1, const float* coef0,
                       float coef0_const, const float* coef1, float coef1_const, int prune, int* offsets, int* columns,
                       float* values, int* bsr_nnz_host, void* workspace, size_t workspace_bytes, gb_stream_t stream);
int gb_q1_assemble_rhs(int dim, int nx, int ny, int nz, int ncomp, const double* M, const float* f, float f0, float f1,
                       float f2, float* out, gb_stream_t stream);
int gb_grid_boundary_mask(int dim, int nx, int ny, int nz, int face_bits, int ncomp, int comp_mask, float* mask,
                          gb_stream_t stream);
int gb_dirichlet_project(int bdim, int nrow, const int* offsets, const int* columns, float* values, const float* mask,
                         float* rhs, const float* fixed, float* tmp, int project_matrix, gb_stream_t stream);

/* ---- Flexible CG preconditioner, multigrid carrier, learned smoother ------------------------------
 * No counterparts in the reference (its only preconditioner is Jacobi, warp/_src/optim/linear.py:236-329).
 * gb_krylov_set_precond: installs z = M(r) for a KRYLOV_FCG handle; fn is called on the host while the
 * solver records its launches (eagerly or into its CUDA graphs) and must enqueue M's kernels on the
 * given stream.  Stagnation (residual not reduced by stag_factor over stag_window iterations, or
 * r.z <= 0) stops the loop with GB_DEV_STAGNATION so the caller can fall back to Jacobi-CG. */
typedef int (*gb_precond_fn)(void* user, gb_stream_t stream, const float* r, float* z);
int gb_krylov_set_precond(void* handle, gb_precond_fn fn, void* user, int stag_window, double stag_factor);
/* Flexible solver with 1x1 blocks: take the product of every iteration from the 27-point stencil form S of
 * the same matrix on an nx x ny x nz node grid (gb_st27_build; the caller keeps S alive); S = NULL returns
 * to the CSR product. */
int gb_krylov_set_stencil(void* handle, int nx, int ny, int nz, const float* S);
/* z_out = z + omega * dinv * (r - A z) (fused Jacobi smoothing step; z_out may not alias z; fp32 or bf16
 * values). */
int gb_bsr_jacobi_smooth(int bdim, int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns,
                         const void* values, int val_dtype, const float* r, const float* z, const float* dinv,
                         float omega, float* z_out, int* status, gb_stream_t stream);
/* Vertex-centred 2:1 transfers on Q1 node grids (nodes per axis; masks 1 = Dirichlet, may be NULL). */
int gb_mg_restrict(int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* r, const float* fmask,
                   const float* cmask, float* rc, gb_stream_t stream);
int gb_mg_prolong_add(int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* zc, const float* fmask,
                      float scale, float* z, gb_stream_t stream);
/* Same transfers for vectors of ncomp (1 or 3) interleaved components per node, node masks. */
int gb_mg_restrict_c(int ncomp, int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* r, const float* fmask,
                     const float* cmask, float* rc, gb_stream_t stream);
int gb_mg_prolong_add_c(int ncomp, int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* zc,
                        const float* fmask, float scale, float* z, gb_stream_t stream);
int gb_mg_jacobi0(int64_t n, float omega, const float* dinv, const float* r, float* z, gb_stream_t stream);
/* Block-Jacobi smoothing of vec3 levels (no reference counterpart): the inverses of the 3x3 diagonal blocks
 * (9 floats per block row, row-major; identity where a block is missing or singular), the first step
 * z_i = omega Dinv_i r_i from zero, and the fused step z_out = z + omega Dinv (r - A z). */
int gb_bsr_block_inverse_diagonal3(int nrow, const int* offsets, const int* row_counts, const int* columns,
                                   const float* values, float* inv, gb_stream_t stream);
int gb_mg_block_jacobi0(int64_t nodes, float omega, const float* dinv_blocks, const float* r, float* z,
                        gb_stream_t stream);
int gb_bsr_block_jacobi_smooth3(int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns,
                                const void* values, int val_dtype, const float* r, const float* z,
                                const float* dinv_blocks, float omega, float* z_out, int* status, gb_stream_t stream);
int gb_mg_coarsen_cells(int fx, int fy, int fz, const float* a, float* ac, gb_stream_t stream);
/* 27-point stencil form of a multigrid level's operator (no reference counterpart): node-major
 * coefficients S[i][k], k = 9(dx+1) + 3(dy+1) + (dz+1), i = (x*ny + y)*nz + z (gb_st27_bytes, 16-byte
 * aligned), built from a compact 1x1 fp32 CSR matrix (status bit 1: an entry outside the
 * 27-neighbourhood).  gb_st27_apply mode 0: out = r - A w;  mode 1: w_out = omega D^-1 r,
 * out = r - A w_out;  mode 2: out = w + omega D^-1 (r - A w); status: GB_DEV_WAIT_TIMEOUT. */
size_t gb_st27_bytes(int nx, int ny, int nz);
int gb_st27_build(int nx, int ny, int nz, const int* offsets, const int* columns, const float* values, float* S,
                  int* status, gb_stream_t stream);
int gb_st27_apply(int mode, int nx, int ny, int nz, const float* S, const float* w, const float* r, const float* dinv,
                  float omega, float* w_out, float* out, int* status, gb_stream_t stream);
/* bf16 copy of S (28 values per node, the last zero; gb_st27_bytes_bf16, 16-byte aligned) and the same
 * three passes reading it, with fp32 accumulation. */
/* r = b - A x on the stencil form S of a 1x1 matrix, x as interleaved (hi, lo) fp32 pairs, double-float
 * arithmetic: gb_residual_df's outputs (r64 / r32 may be null; norms = ||r||^2, ||b||^2) and workspace
 * (gb_residual_f64_workspace_bytes; its first 256 bytes an arrival counter, zero before the first call). */
int gb_residual_df_st27(int nx, int ny, int nz, const float* S, const void* x2, const float* b, double* r64,
                        float* r32, double* norms, void* workspace, size_t workspace_bytes, int* status,
                        gb_stream_t stream);
size_t gb_st27_bytes_bf16(int nx, int ny, int nz);
int gb_st27_to_bf16(int nx, int ny, int nz, const float* S, void* Sb, gb_stream_t stream);
int gb_st27_apply_bf16(int mode, int nx, int ny, int nz, const void* Sb, const float* w, const float* r,
                       const float* dinv, float omega, float* w_out, float* out, int* status, gb_stream_t stream);
/* 3x3x3 convolutions on a node grid, channels-last activations act[v][C], v = (x*ny + y)*nz + z,
 * weights W[t][ci][co] (t = 9(dx+1) + 3(dy+1) + (dz+1)), zero padding.  fp32 training kernels
 * (gb_conv3_bwd_weight_f32 accumulates into gW, deterministic), Adam, features and the combine step
 * of the training forward. */
int gb_conv3_fwd_f32(int nx, int ny, int nz, int cin, int cout, const float* in, const float* W, int relu, float* out,
                     gb_stream_t stream);
int gb_conv3_bwd_data_f32(int nx, int ny, int nz, int cin, int cout, const float* gout, const float* W, float* gin,
                          gb_stream_t stream);
size_t gb_conv3_bwd_weight_workspace_bytes(int nx, int ny, int nz, int cin, int cout);
int gb_conv3_bwd_weight_f32(int nx, int ny, int nz, int cin, int cout, const float* in, const float* gout, float* gW,
                            void* workspace, size_t workspace_bytes, gb_stream_t stream);
int gb_relu_bwd(int64_t n, const float* out, float* g, gb_stream_t stream);
int gb_adam_step(int n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps, int step,
                 void* w_bf16, gb_stream_t stream);
int gb_net_features(int dtype, int ncomp, int64_t n, const float* r, const float* dinv, const float* chat,
                    const float* mask, void* out, gb_stream_t stream);
int gb_net_cell_features(int nx, int ny, int nz, const float* cell_coef, float mean_log, float inv_std, float* chat,
                         gb_stream_t stream);
int gb_net_combine(int dtype, int ncomp, int64_t n, int stride, const void* act, const float* mask, float omega,
                   const float* dinv, const float* r, float* out, gb_stream_t stream);
/* tcgen05 implicit-GEMM layers on the planar padded layout: the grid padded by one zero voxel per side,
 * row p = ((x+1)(ny+2) + (y+1))(nz+2) + (z+1), channels 0-7 in plane 0 and 8-15 in plane 1 (16 B per row),
 * planes gb_conv3_planar_rows() rows apart, border rows zero.  last = 0: ReLU layer, planar bf16 out;
 * last = 1: w = omega dinv r + (mask ? 0 : channel 0) in fp32; last = 3 (vec3 fields, 3 interleaved dofs per
 * node): w[3v+c] = omega dinv[3v+c] r[3v+c] + (mask[v] ? 0 : channel c).  Wt: [27][16][16] bf16.
 * Features (gb_net_features*): ncomp = 1 scalar fields (x = dinv r and x times the 8 adjacent cells'
 * normalised log-coefficients), ncomp = 3 vec3 fields (x_c and x_c times the mean and x/y/z contrasts of
 * those 8 values).  gb_net_combine: out[dof] = omega dinv r + (mask[node] ? 0 : act[node][c]). */
int64_t gb_conv3_planar_rows(int nx, int ny, int nz);
int gb_net_features_planar(int ncomp, int nx, int ny, int nz, const float* r, const float* dinv, const float* chat,
                           const float* mask, void* out, gb_stream_t stream);
int gb_conv3_fwd_tc(int nx, int ny, int nz, int last, const void* in, const void* Wt, void* out, float* w,
                    const float* r, const float* dinv, const float* mask, float omega, int* status, gb_stream_t stream);
/* The whole network (features, nlayers - 1 ReLU layers, the last layer into w as last = ncomp) in one
 * cooperative launch: act[l] is layer l's planar input (act[0] the features), flags holds
 * gb_convnet_tc_items() uint32 counters and epoch 2 uint32, all zero before the first launch and shared only
 * by consecutive launches of the same nlayers on one stream.  GB_ERR_UNSUPPORTED (nothing launched) when the
 * device cannot hold every CTA at once. */
int64_t gb_convnet_tc_items(int nx, int ny, int nz);
int gb_convnet_fwd_tc(int nx, int ny, int nz, int ncomp, int nlayers, void* const* act, const void* const* Wt,
                      float* w, const float* r, const float* dinv, const float* chat, const float* mask, float omega,
                      unsigned int* flags, unsigned int* epoch, int* status, gb_stream_t stream);

/* Multi-column dot / axpy for GMRES's Gram-Schmidt steps (warp/_src/optim/linear.py:1653-1916 computes
 * them with TiledDot over the basis and _gmres_arnoldi_axpy_kernel): out[c] = V[c] . w (rows of V ldv
 * apart, fp64 accumulation, deterministic); w = beta w + alpha sum_c coef[c] V[c] (coef: device doubles). */
size_t gb_multi_dot_workspace_bytes(int ncols);
int gb_multi_dot(int dtype, int64_t n, int ncols, const void* V, int64_t ldv, const void* w, double* out,
                 void* workspace, size_t workspace_bytes, gb_stream_t stream);
int gb_multi_axpy(int dtype, int64_t n, int ncols, const void* V, int64_t ldv, const double* coef, double alpha,
                  double beta, void* w, gb_stream_t stream);

/* ---- Row-local compression (the "row_compress" construction) ------------------------------------
 * gb_bsr_compress_rows replaces bsr_compress(inplace=True) (warp/_src/sparse.py:1571-1640 ->
 * warp/native/sparse.cu:1494-1656, per-row routine warp/native/sparse_util.h:82-139): prune zero
 * blocks, stable sort by column and coalesce each active row in place, out_counts[r] = blocks kept.
 * gb_bsr_compact: compact CSR (exclusive scan of counts[nrow + 1], counts[nrow] = 0, then a gather).
 * gb_bsr_rows_to_offsets: padded row starts of candidates grouped by row (fem.integrate assembles
 * them that way, warp/_src/fem/integrate.py:1664-1712); unsorted or out-of-range rows set status. */
int gb_bsr_rows_to_offsets(int64_t T, const int* rows, int nrow, int* offsets, int* status, gb_stream_t stream);
int gb_bsr_compress_rows(int block_size, int dtype, int nrow, const int* offsets, const int* row_counts, int* columns,
                         void* values, int prune, uint64_t zero_mask, int* out_counts, gb_stream_t stream);
size_t gb_bsr_compact_workspace_bytes(int nrow);
int gb_bsr_compact(int block_size, int dtype, int nrow, const int* old_offsets, int* counts, const int* columns_in,
                   const void* values_in, int* offsets_out, int* columns_out, void* values_out, void* workspace,
                   size_t workspace_bytes, gb_stream_t stream);

/* ---- Padded topology of bsr_set_from_triplets --------------------------------------------------
 * gb_bsr_scatter_padded replaces _bsr_set_from_triplets_padded_scatter_compact_topology
 * (warp/_src/sparse.py:1173-1208): copy each row of a compact structure into the destination's row
 * capacity [dest_offsets[r], dest_offsets[r+1]); rows that do not fit get dest_row_counts[r] = 0 and
 * raise *status to 1 (BSR_STATUS_ROW_CAPACITY_EXCEEDED, atomic max); block_map (optional) receives,
 * per padded slot, the compact block it holds or -1.
 * gb_bsr_gather_blocks: dst[b] = src[block_map[b]] or 0 for -1 (the value pass of the padded
 * topology, warp/_src/sparse.py:1211-1230, applied to the compact run sums). */
int gb_bsr_scatter_padded(int nrow, const int* compact_offsets, const int* compact_columns, const int* dest_offsets,
                          int* dest_row_counts, int* dest_columns, int* block_map, int* status, gb_stream_t stream);
int gb_bsr_gather_blocks(int dtype, int block_size, int64_t nblocks, const int* block_map, const void* src, void* dst,
                         gb_stream_t stream);

/* ---- Batched solves --------------------------------------------------------------------------
 * gb_batched_pcg replaces the batched CG of warp/_src/optim/linear.py:893-1032 (LinearOperator with
 * batch_offsets, :33-133; per-subproblem tolerances :2063-2083; frozen converged subproblems
 * :2333-2373) for a block-diagonal compact CSR (1x1 BSR) fp32 matrix with Jacobi (dinv) or no
 * preconditioner: one persistent launch in which each CTA -- or, for subproblems of at most small_rows
 * rows, each warp -- runs one subproblem's CG to its own convergence, taking subproblems from a queue
 * in the order `order` (largest first).  Rows >= batch_offsets[nbatch] are not touched.
 * threads: 128/256/512/1024; lanes_per_row: 1/2/4/8; grid <= 0: automatic.
 * gb_q1_batched_assemble_2d: block-diagonal Q1 diffusion systems on unit squares (no reference
 * counterpart: the reference assembles each subproblem with fem.integrate). */
size_t gb_batched_pcg_workspace_bytes(int64_t n);
int gb_batched_pcg(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                   const int* columns, const float* values, const float* dinv, const float* b, float* x, double rtol,
                   double atol, int maxiter, int x_is_zero, int threads, int lanes_per_row, int small_rows, int grid,
                   int* iters, float* rr, float* atol_sq, void* workspace, size_t workspace_bytes, int* status,
                   gb_stream_t stream);
/* Same solve; smem_rows > 0: CTA-mode subproblems of at most smem_rows rows keep p, r, Ap in shared
 * memory (3 * 4 * smem_rows bytes per CTA, at most 200 KB; results identical to smem_rows = 0). */
int gb_batched_pcg2(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                    const int* columns, const float* values, const float* dinv, const float* b, float* x, double rtol,
                    double atol, int maxiter, int x_is_zero, int threads, int lanes_per_row, int small_rows,
                    int smem_rows, int grid, int* iters, float* rr, float* atol_sq, void* workspace,
                    size_t workspace_bytes, int* status, gb_stream_t stream);
/* gb_batched_bicgstab replaces BiCGSTAB with batch_offsets (warp/_src/optim/linear.py:1377-1574; per-subproblem
 * tolerances :2063-2083): the same persistent queue of subproblems, one CTA per subproblem running its
 * BiCGSTAB (right preconditioning, left with left_precond; Jacobi dinv or none) to its own tolerance.
 * Workspace: gb_batched_bicgstab_workspace_bytes(n) (8 work vectors). */
size_t gb_batched_bicgstab_workspace_bytes(int64_t n);
int gb_batched_bicgstab(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                        const int* columns, const float* values, const float* dinv, const float* b, float* x,
                        double rtol, double atol, int maxiter, int x_is_zero, int left_precond, int threads,
                        int lanes_per_row, int grid, int* iters, float* rr, float* atol_sq, void* workspace,
                        size_t workspace_bytes, int* status, gb_stream_t stream);
int gb_q1_batched_assemble_2d(int nbatch, const int* ncell, const int* row_off, const int* nnz_off,
                              const int* cell_off, const float* coef, const float* f, int total_rows, int* offsets,
                              int* columns, float* values, float* rhs, gb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* WARP_GB300_H */
