/*
 * tfcuda.h -- C ABI of libtfcuda.so, the GB300 (sm_103a) backend of the
 * TransiFlow finite-volume hot path.
 *
 * Conventions
 *   - Every device buffer is allocated by the caller (the Python host layer
 *     uses PyTorch's caching allocator).  Functions never allocate or free;
 *     scratch needs are reported by *_workspace_bytes queries.
 *   - Pointers named d_* are device pointers; everything else is host memory.
 *   - All work is enqueued on the given stream (0 = legacy default stream)
 *     and is stream ordered; functions return before the GPU finishes.
 *   - Return value: TF_OK (0) or a positive TF_ERR_* code; tf_error_string()
 *     describes it.  Non-convergence of an iterative method is reported
 *     through output arguments, never by a trap.
 *   - State vectors are interleaved per cell, [u, v, (w), p, (T)] with x
 *     fastest: index = d + dof * (i + nx * (j + ny * k)), as in
 *     transiflow/utils.py:23-60 (create_state_mtx).
 *
 * Reference interfaces replaced (BIMAU/transiflow 1.0.1):
 *   tf_assemble         Discretization.rhs / jacobian, Discretization.py:367-415
 *                       (+ nonlinear_part :319-365, linear_part :210-317,
 *                       boundaries :704-714, assemble_rhs :439-472,
 *                       assemble_jacobian :474-524)
 *   tf_stencil_pattern  the column structure of assemble_jacobian, :507-522
 *   tf_csr_compact      CrsMatrix.compress, CrsMatrix.py:52-71
 *   tf_mass_diag        Discretization.mass_matrix, Discretization.py:417-548
 *   tf_gauge_values     SciPy.Interface.compute_bordered_matrix pressure fix,
 *                       interface/SciPy.py:93-103
 *   tf_spmv_*           scipy CSC @ and CrsMatrix.matvec, CrsMatrix.py:155-170
 *   tf_nd_*             splu / lu.solve, interface/SciPy.py:151, 194-202
 *   tf_vec_*            vector algebra used by Continuation.py and by the
 *                       GMRES that replaces scipy.sparse.linalg.gmres
 */
#ifndef TFCUDA_H
#define TFCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *tf_stream_t;

enum {
    TF_OK = 0,
    TF_ERR_ARG = 1,          /* invalid argument (null pointer, bad size)   */
    TF_ERR_UNSUPPORTED = 2,  /* (dim, dof) combination not compiled in      */
    TF_ERR_CUDA = 3,         /* a CUDA launch or runtime call failed        */
    TF_ERR_SIZE = 4,         /* a size exceeds a compiled-in maximum        */
    TF_ERR_TIMEOUT = 5       /* a bounded device-side wait gave up          */
};

/* ---- problem description -------------------------------------------------*/

#define TF_MAX_BC_OPS 24

enum { TF_BC_WALL = 1, TF_BC_FORCE = 2, TF_BC_FORCE_PROFILE = 3, TF_BC_PIN = 4 };

/* One boundary-condition primitive applied to the atoms of the cells on one
 * face of the box (BoundaryConditions.py:55-544):
 *   TF_BC_WALL : no-slip (sign = -1) or free-slip (sign = +1) wall,
 *                BoundaryConditions.py:55-233;
 *   TF_BC_FORCE: _constant_forcing_* with forcing constant fc and atom
 *                constant ac for variable var, BoundaryConditions.py:471-544
 *                (moving lids, fixed temperatures, heat and salinity fluxes
 *                reduce to this);
 *   TF_BC_FORCE_PROFILE: the same with a forcing that varies along the
 *                face (2D only): the neighbour at tangential index m (m = -1
 *                is the ghost before the first cell) is forced by
 *                d_prof[row * prof_len + (m < 0 ? prof_len - 1 : m)] with
 *                row = (int)fc, as numpy.ones((n + 2, .)) * value indexes it;
 *   TF_BC_PIN  : fix one value of variable var (Discretization.py:690-702):
 *                every entry coupling to var of cell (0,0,0), periodic
 *                neighbours included, becomes 0, that row gets -1 on its
 *                diagonal and no forcing.  Applied in op order, i.e. last.   */
typedef struct tf_bc_op {
    int32_t kind;
    int32_t axis;   /* 0 = x, 1 = y, 2 = z                */
    int32_t high;   /* 1 = east/north/top, 0 = west/...   */
    int32_t var;    /* WALL: sign (+1/-1); FORCE: variable */
    double fc;
    double ac;
} tf_bc_op;

/* Scalars of Discretization._linear_part_2D/3D (Discretization.py:229-317)
 * and the boundary program, plus the per-axis metric table.
 * metric: device pointer to double[3][TF_METRIC_FIELDS][metric_stride] with
 * fields, for cell m of face coordinates c:
 *   D = c[m]-c[m-1], Dp = c[m+1]-c[m], H = (c[m]-c[m-2])/2,
 *   Hp = (c[m+1]-c[m-1])/2, rD = 1/D, rDp = 1/Dp, rH = 1/H, rHp = 1/Hp,
 *   w0 = 1/2*D/Hp, w1 = 1/2*Dp/Hp.                                          */
#define TF_METRIC_FIELDS 10

typedef struct tf_problem {
    int32_t nx, ny, nz, dim, dof;
    int32_t nonlinear;     /* 0 when Re == 0 and there is no temperature     */
    int32_t buoy_row;      /* velocity row with the buoyancy term, -1 none   */
    int32_t biot_row;      /* velocity column of the Biot term, -1 none      */
    double visc;           /* 1 / (Re * sqrt(Gr))                            */
    double cond;           /* 1 / (Pr * sqrt(Gr))                            */
    double biot;           /* Bi / (Bi + 1)                                  */
    const double *d_metric;
    int32_t metric_stride;
    int32_t nops;
    tf_bc_op ops[TF_MAX_BC_OPS];
    /* beta-plane Coriolis term and wind stress (2D; Discretization.py:253-255,
     * 1086-1118): rossby = 'Rossby Parameter' (0: no Coriolis term), wind =
     * 'Wind Stress Parameter' / (2 pi) (0: no wind forcing), asym = 'Asymmetry
     * Parameter'.  d_aux: device pointer to double[4][ny] with, for row j of
     * face coordinates y: y[j]/2, -(y[j]+y[j-1])/4, cos(2 pi yc), cos(pi yc),
     * yc = (y[j]+y[j-1])/2; may be NULL when rossby == wind == 0.             */
    double rossby;
    double wind;
    double asym;
    const double *d_aux;
    /* salinity (dof = dim + 3): sal = 1 / (Le * Pr * sqrt(Gr))
     * (Discretization.py:260-263); d_prof / prof_len: the forcing profiles of
     * TF_BC_FORCE_PROFILE ops, nprof profiles of prof_len values (NULL / 0 if
     * none). */
    double sal;
    const double *d_prof;
    int32_t prof_len;
    int32_t nprof;         /* number of profiles in d_prof                   */
} tf_problem;

/* ---- library ------------------------------------------------------------*/

int tf_version(void);
const char *tf_error_string(int code);
/* Number of kernel launches (and device memsets) the library has issued
 * since load or the last reset; host-side counter, no synchronisation.      */
long long tf_launch_count(void);
void tf_launch_count_reset(void);
/* A non-blocking stream owned by the caller (never shared, unlike pooled
 * streams: concurrent instances capture CUDA graphs on their own streams). */
int tf_stream_create(tf_stream_t *out);
int tf_stream_destroy(tf_stream_t stream);

/* ---- stencil CSR ----------------------------------------------------------
 * The Jacobian is stored as a CSR whose rows have a fixed width per
 * variable: every cell stores, for each of its dof rows, the structural
 * superset of the reference's entries (all (d2, offset) an atom can hold),
 * sorted by column.  Entries whose neighbour cell lies outside the grid are
 * kept as zeros with a clamped column.  Row r = cell*dof + d1 starts at
 * cell*width + row_offset[d1].                                              */

/* Host query: cell width and per-variable row offsets (dof + 1 ints) and the
 * slot table slot[(d1*dof + d2)*27 + ox + 3*oy + 9*oz] (-1: not stored).    */
int tf_stencil_layout(int dim, int dof, int *row_offset, int *slot);

/* rowptr[n+1] and cols[nnz] of the stencil CSR for the grid of p.          */
int tf_stencil_pattern(const tf_problem *p, int32_t *d_rowptr, int32_t *d_cols,
                       tf_stream_t stream);

/* Fused assembly: F(x) into d_rhs and/or the Jacobian values into d_jvals
 * (either may be NULL).  Bit-compatible with the reference's floating-point
 * operation order.  Values with |v| <= 1e-14 are stored as 0.                */
int tf_assemble(const tf_problem *p, const double *d_state, double *d_rhs,
                double *d_jvals, tf_stream_t stream);

/* Diagonal of the mass matrix (pressure entries 0).                          */
int tf_mass_diag(const tf_problem *p, double *d_diag, tf_stream_t stream);

/* Export to the reference's compressed CSR: drop zeros, merge duplicate
 * columns in stored order (CrsMatrix.compress).  Two passes: call with
 * d_out_cols == NULL to get d_out_rowptr (n+1) and *nnz (host), then again
 * with output arrays of that size.                                           */
int tf_csr_compact(int n, const int32_t *d_rowptr, const int32_t *d_cols,
                   const double *d_vals, int32_t *d_out_rowptr, int32_t *d_out_cols,
                   double *d_out_vals, int64_t *nnz, void *d_work, size_t work_bytes,
                   tf_stream_t stream);
size_t tf_csr_compact_workspace_bytes(int n);

/* Copy of d_vals with the pressure gauge applied (row and column g replaced
 * by a single -1 on the diagonal), as the SciPy backend does before splu.   */
int tf_gauge_values(int n, const int32_t *d_rowptr, const int32_t *d_cols,
                    const double *d_vals, int gauge, double *d_out, tf_stream_t stream);

/* y = alpha * A x + beta * y (beta == 0: y is not read).                     */
int tf_spmv_f64(int n, const int32_t *d_rowptr, const int32_t *d_cols,
                const double *d_vals, const double *d_x, double *d_y,
                double alpha, double beta, tf_stream_t stream);
int tf_spmv_f32(int n, const int32_t *d_rowptr, const int32_t *d_cols,
                const float *d_vals, const double *d_x, double *d_y,
                double alpha, double beta, tf_stream_t stream);

/* Equilibration before a low-precision factorisation (no counterpart in the
 * reference, whose SuperLU factors in FP64): row scales d_rscale[i] and
 * column scales d_cscale[j], powers of two near 1 / max |entry| of the row
 * and then of the row-scaled column (1 for empty ones), and d_out[k] =
 * d_rscale[row] * d_vals[k] * d_cscale[col] (d_out may alias d_vals).  The
 * preconditioner of A is then d_cscale .* (LU of d_out)^-1 (d_rscale .* b).  */
int tf_equilibrate(int n, const int32_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                   double *d_rscale, double *d_cscale, double *d_out, tf_stream_t stream);
/* y[i] = d[i] * x[i] (y may alias x).                                         */
int tf_vec_mul(int n, const double *d_d, const double *d_x, double *d_y, tf_stream_t stream);
/* y[i] += a * diag[i] * x[i] (diagonal matrix product used by theta-method
 * residuals and J - M / (theta dt)).                                         */
int tf_diag_axpy(int n, double a, const double *d_diag, const double *d_x, double *d_y,
                 tf_stream_t stream);
/* vals[diag slot of row r] += a * diag[r] for every row with a stored
 * diagonal (rows of the stencil CSR always store one).                      */
int tf_add_diagonal(int n, const int32_t *d_rowptr, const int32_t *d_cols, double *d_vals,
                    double a, const double *d_diag, tf_stream_t stream);

/* ---- dense vector kernels (GMRES, continuation) -------------------------*/

/* out[j] = sum_i V[j*ldv + i] * w[i] for j < k  (k <= 256); deterministic
 * two-pass reduction; out is device memory.                                  */
int tf_vec_mdot(int n, int k, const double *d_V, long long ldv, const double *d_w,
                double *d_out, void *d_work, size_t work_bytes, tf_stream_t stream);
size_t tf_vec_mdot_workspace_bytes(int n, int k);
/* Same result as tf_vec_mdot, for callers that cannot allocate device
 * memory (no counterpart in the reference): a host application that gives
 * the library a fixed device-memory budget and forbids further cudaMalloc,
 * or a loop that must not incur the device-wide synchronisation of
 * cudaMalloc/cudaFree.  The partial sums live in a fixed 152 KiB device array
 * inside the library that every GPU loading it holds until exit; nothing is
 * allocated per call.  k must not exceed 64 (TF_ERR_SIZE otherwise).  The
 * first call on a device looks up the array's device address with that
 * device current and keeps it for the life of the process; make that first
 * call before any stream capture.  After cudaDeviceReset on a device the
 * kept address is stale: a process that resets a device must not call this
 * entry point on it again.  All calls share the array: calls that overlap on
 * the GPU race.                                                             */
int tf_vec_mdot_noalloc(int n, int k, const double *d_V, long long ldv, const double *d_w,
                        double *d_out, tf_stream_t stream);
/* w[i] -= sum_j V[j*ldv+i] * h[j]  (h device, k <= 256)                     */
int tf_vec_mgs_update(int n, int k, const double *d_V, long long ldv, const double *d_h,
                      double *d_w, tf_stream_t stream);
/* z = a x + b y (x or y may be NULL, meaning absent; z may alias x or y).    */
int tf_vec_axpby(int n, double a, const double *d_x, double b, const double *d_y,
                 double *d_z, tf_stream_t stream);
/* z = x / s, IEEE division per element (z may alias x).                      */
int tf_vec_div(int n, const double *d_x, double s, double *d_z, tf_stream_t stream);
/* d_z *= 1 / sqrt(*d_nrm2) with the square norm read on the device (the
 * normalisation of an Arnoldi vector without a host round trip).            */
int tf_vec_scale_rsqrt(int n, const double *d_nrm2, double *d_z, tf_stream_t stream);
int tf_vec_fill(int n, double a, double *d_z, tf_stream_t stream);
int tf_vec_to_f32(int n, const double *d_x, float *d_y, tf_stream_t stream);

/* ---- nested-dissection multifrontal LU (tf_nd.cu) ------------------------*/

typedef struct tf_nd_plan {
    int32_t n;            /* unknowns                                        */
    int32_t nnodes;
    int32_t nlevels;
    const int32_t *level_ptr;   /* host: nodes of height h are              */
                                /* [level_ptr[h], level_ptr[h+1])            */
    const int32_t *max_own;     /* host: per level max own size              */
    const int32_t *max_f;       /* host: per level max front size            */
    const int32_t *d_n_own;
    const int32_t *d_f;
    const int32_t *d_parent;
    const int64_t *d_front_off; /* nnodes + 1                                */
    const int64_t *d_idx_off;   /* nnodes + 1                                */
    const int32_t *d_idx;       /* own then boundary unknowns per node        */
    const int64_t *d_ea_off;    /* nnodes + 1                                */
    const int32_t *d_ea_map;    /* child boundary -> parent front position   */
    int64_t nscat;
    const int64_t *d_scat_pos;  /* front element receiving each entry         */
    const int32_t *d_scat_src;  /* stencil-CSR entry index                    */
    const int64_t *scat_level_ptr; /* host: entries of level h               */
    const int64_t *d_piv_off;   /* nnodes + 1: pivot storage offsets (own)    */
    const int32_t *d_rank;      /* 0/1: position among the parent's children  */
    int64_t front_elems;        /* total front elements                       */
    /* FP32 factorisations: tree heights whose widest front has at least this
     * many rows are factored in outer blocks of 256 columns, each followed by
     * one rank-256 trailing update on the tensor cores (tcgen05, TF32
     * products, FP32 sums); 0 keeps rank-32 FP32 updates everywhere.        */
    int32_t tc_min_front;
    /* products of those updates: 1 = one TF32 product per term, 3 (or any
     * other value) = operands split into TF32 high parts and remainders,
     * three products per term, close to FP32 accuracy                        */
    int32_t tc_terms;
    /* FP32 / BF16 applications: warps per SM a height's launch aims for
     * before a warp takes fewer column tiles (0: 64).  Tuned at run time by
     * the Python solver ('Tune Application'); any value gives the same
     * results up to the order of the atomic sums.                          */
    int32_t apply_waves;
} tf_nd_plan;

/* Numeric factorisation of the (gauged) stencil-CSR values.  d_fronts holds
 * plan->front_elems elements of the factor precision; d_piv holds plan->n
 * int32.  d_info (device int32, may be NULL) is incremented once per exactly
 * zero pivot (the pivot is then replaced by 1e-30 and the solve is useless).*/
int tf_nd_factor_f64(const tf_nd_plan *plan, const double *d_vals, double *d_fronts,
                     int32_t *d_piv, int32_t *d_info, tf_stream_t stream);
int tf_nd_factor_f32(const tf_nd_plan *plan, const double *d_vals, float *d_fronts,
                     int32_t *d_piv, int32_t *d_info, tf_stream_t stream);
/* One rank-w tensor-core trailing update of every front of tree height
 * `height`: F[r][j] -= L[r][k0:E] U[k0:E][j] for r, j >= E = min(k0 + 256,
 * n_own), FP32 fronts, TF32 products (terms = 1, or 3 for split operands)
 * with FP32 accumulation (the step the
 * FP32 factorisation runs after each outer block; exposed for tests).
 * Needs only d_n_own, d_f, d_front_off, level_ptr, max_f and nlevels of the
 * plan.  No counterpart in the reference (SuperLU, SciPy.py:151).          */
int tf_nd_tc_update_f32(const tf_nd_plan *plan, int height, int k0, int terms, float *d_fronts,
                        int32_t *d_info, tf_stream_t stream);
/* In-place solve of the factored system: d_x (length n, FP64) holds the
 * right-hand side on entry and the solution on exit.  The f32 variant works
 * in single precision on the FP64 vector.                                    */
int tf_nd_solve_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv,
                    double *d_x, tf_stream_t stream);
int tf_nd_solve_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv,
                    double *d_x, tf_stream_t stream);

/* Replaces, in place, the factored own blocks L11 and U11 of every front by
 * their inverses (recursive halving, batched GEMMs), so that tf_nd_solve_inv_*
 * applies the factors without sequential substitution.  Call after
 * tf_nd_factor_* on the same fronts; the fronts are then usable only with
 * tf_nd_solve_inv_*.  d_work: tf_nd_invert_workspace_bytes(plan, sizeof
 * element) bytes of device scratch.  No counterpart in the reference (its
 * SuperLU solve substitutes, SciPy.py:194-202).                              */
size_t tf_nd_invert_workspace_bytes(const tf_nd_plan *plan, int elem_size);
int tf_nd_invert_f64(const tf_nd_plan *plan, double *d_fronts, double *d_work, size_t work_bytes,
                     tf_stream_t stream);
int tf_nd_invert_f32(const tf_nd_plan *plan, float *d_fronts, float *d_work, size_t work_bytes,
                     tf_stream_t stream);
/* tf_nd_factor_* followed by tf_nd_invert_*, with the inversion of each tree
 * height's own blocks on aux_stream as soon as that height is factored, so
 * that it overlaps the factorisation of the heights above.  aux_stream must
 * differ from stream and is joined back into stream before the call returns
 * (also inside a stream capture: the pair becomes one graph).               */
int tf_nd_factor_inv_f64(const tf_nd_plan *plan, const double *d_vals, double *d_fronts, int32_t *d_piv,
                         int32_t *d_info, double *d_work, size_t work_bytes, tf_stream_t stream,
                         tf_stream_t aux_stream);
int tf_nd_factor_inv_f32(const tf_nd_plan *plan, const double *d_vals, float *d_fronts, int32_t *d_piv,
                         int32_t *d_info, float *d_work, size_t work_bytes, tf_stream_t stream,
                         tf_stream_t aux_stream);
/* In-place solve with inverted own blocks (after tf_nd_invert_*): d_x as in
 * tf_nd_solve_*; d_scratch: tf_nd_solve_inv_workspace_bytes(plan) bytes of
 * device scratch, the larger of one double per front index entry (FP64
 * factors) and 2 n doubles (FP32 / BF16 factors: the vectors y and z of the
 * application, addressed by unknown); the query reads the plan's last index
 * offset from the device, a synchronising copy.  Replaces SuperLU's solve
 * in SciPy.Interface.direct_solve (transiflow/interface/SciPy.py:204-258). */
size_t tf_nd_solve_inv_workspace_bytes(const tf_nd_plan *plan);
int tf_nd_solve_inv_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv,
                        double *d_x, double *d_scratch, tf_stream_t stream);
int tf_nd_solve_inv_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv,
                        double *d_x, double *d_scratch, tf_stream_t stream);
/* BF16 storage of an FP32 factorisation for its applications: the factor
 * entries an application reads (every own row; the own columns of the
 * boundary rows) of the inverted FP32 fronts, rounded to BF16 into d_out,
 * which has the fronts' layout (plan->front_elems 2-byte elements; entries
 * an application does not read are left as they are).  Call after
 * tf_nd_factor_inv_f32 / tf_nd_invert_f32.  tf_nd_solve_inv_bf16 applies
 * them with FP32 products and sums (d_x, d_scratch as for
 * tf_nd_solve_inv_f32), reading half the bytes of the FP32 application.
 * No counterpart in the reference (SuperLU keeps FP64 factors,
 * SciPy.py:151).                                                            */
int tf_nd_factors_to_bf16(const tf_nd_plan *plan, const float *d_fronts, uint16_t *d_out, tf_stream_t stream);
int tf_nd_solve_inv_bf16(const tf_nd_plan *plan, const uint16_t *d_fronts, const int32_t *d_piv,
                         double *d_x, double *d_scratch, tf_stream_t stream);

/* The same application as tf_nd_solve_inv_* in ONE persistent launch: both
 * sweeps run as a task list over the elimination tree, each task waiting
 * (bounded) only for the fronts it depends on.  Setup, once per plan:
 * tf_nd_flow_workspace_bytes (0 on a bad plan) and tf_nd_flow_prepare, both
 * synchronising (they read the plan's front sizes from the device).
 * elem_size: 8 (f64 fronts) or 4 (f32); TF_ERR_SIZE when the plan's widest
 * front does not fit the launch's shared memory (use tf_nd_solve_inv_*).
 * fuse_tiles: fronts with at most this many 32x32 factor tiles per sweep run
 * as one task (0: never); chunk_tiles: target tiles per task of the others.
 * d_work is then passed to every solve (one application at a time per
 * workspace).  tf_nd_flow_status returns and clears the sticky error word:
 * TF_ERR_TIMEOUT when a wait gave up (the solution is then invalid), a
 * synchronising read.  No counterpart in the reference (SciPy.py:194-202
 * substitutes with SuperLU's factors).                                       */
size_t tf_nd_flow_workspace_bytes(const tf_nd_plan *plan, int fuse_tiles, int chunk_tiles);
int tf_nd_flow_prepare(const tf_nd_plan *plan, void *d_work, size_t work_bytes, int elem_size,
                       int fuse_tiles, int chunk_tiles);
int tf_nd_solve_flow_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv,
                         double *d_x, void *d_work, tf_stream_t stream);
int tf_nd_solve_flow_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv,
                         double *d_x, void *d_work, tf_stream_t stream);
int tf_nd_flow_status(void *d_work);
/* Host-only: the task list tf_nd_flow_prepare builds, from host copies of the
 * plan's per-front own sizes, front sizes and parents and its level_ptr.
 * tasks: 8 int32 per task (front, kind, first row, end row, counter waited
 * for or -1, target count, counter signalled or -1, 0); nodes: 8 int32 per
 * front (forward wait, target, signal, backward wait, target, signal, 0, 0),
 * read by the one-warp tasks of small fronts (kinds 5 forward, 6 backward,
 * front range [front, front + first row)).  With tasks or nodes NULL only
 * *ntasks is set.  No device memory is touched.                             */
int tf_nd_flow_tasks_host(int nnodes, const int32_t *n_own, const int32_t *f, const int32_t *parent,
                          int nlevels, const int32_t *level_ptr, int fuse_tiles, int chunk_tiles,
                          int32_t *tasks, int32_t *nodes, int max_tasks, int *ntasks);

/* ---- learned continuation predictor ---------------------------------------
 * A stack of 3x3x3 convolutions over the cell grid proposing the correction
 * to the secant predictor (x0 + ds*t) of pseudo-arclength continuation; the
 * reference has only the secant predictor (transiflow/Continuation.py:
 * 258-260), so these entry points replace none of its interfaces.
 * Activations are channels-last BF16 [cell][kp], cell = i + nx*(j + ny*k);
 * kp and np (channels in and out) are 16 or 32.  Weights: forward layout
 * BF16 [27][np][kp]; backward-data layout BF16 [27][kp][np] holding the
 * mirrored tap (26 - tap); FP32 master weights [27][kp][np] and bias [np];
 * gradients and Adam moments FP32 [28][kp][np] (slot 27, row 0: the bias).
 *
 * tf_sg_conv: Z = conv(X, W) + bias (FP32 [cell][np], nullable) and A =
 *   relu(Z) if relu else Z (BF16 [cell][np], nullable; not both null);
 *   d_bias may be null (no bias).  With the backward-data weights and dZ as
 *   X it computes the gradient with respect to the layer's input.
 * tf_sg_wgrad: grad (+)= d loss / d (w, bias) from the layer input X (BF16
 *   [cell][kp]) and dZ (FP32 [cell][np]); a per-chunk partial sum in d_work
 *   (tf_sg_wgrad_workspace_bytes), reduced in a fixed order.
 * tf_sg_loss: loss[0] = mean over cells and the first dof channels of
 *   (out - tgt)^2, with dZ = d loss / d out in FP32 and BF16; d_work:
 *   tf_sg_loss_workspace_bytes.
 * tf_sg_act_grad: dZ = dA where Z > 0 else 0, FP32 and BF16 (n elements).
 * tf_sg_pack: the network input from the FP64 state x and tangent t (scaled
 *   by the host arrays sx, st of dof entries), optionally a third field p
 *   (d_p, scaled by sp; NULL: none), then the parameter mu and step ds.
 * tf_sg_target: tgt = (x1 - x0 - ds t) * inv_scale[d] (FP32).
 * tf_sg_unpack: xp = x0 + ds t + scale[d] * out[cell][d] (FP64); entries
 *   whose tangent t is exactly zero (unknowns the branch does not move, such
 *   as the pressure gauge) get x0 + ds t only.
 * tf_sg_adam: one Adam step (step >= 1, bias-corrected) of the master
 *   weights with the gradient scaled by grad_scale, then both BF16 layouts;
 *   step 0 only writes the BF16 layouts (d_grad, d_m, d_v may be null).    */
int tf_sg_conv(int nx, int ny, int nz, int kp, int np, const void *d_x, const void *d_w, const float *d_bias,
               float *d_z, void *d_a, int relu, tf_stream_t stream);
size_t tf_sg_wgrad_workspace_bytes(int ncell, int kp, int np);
int tf_sg_wgrad(int nx, int ny, int nz, int kp, int np, const void *d_x, const float *d_dz, float *d_grad,
                int accumulate, void *d_work, size_t work_bytes, tf_stream_t stream);
size_t tf_sg_loss_workspace_bytes(int ncell, int np);
int tf_sg_loss(int ncell, int dof, int np, const float *d_out, const float *d_tgt, float *d_dzf, void *d_dzh,
               double *d_loss, void *d_work, size_t work_bytes, tf_stream_t stream);
int tf_sg_act_grad(long long n, const float *d_da, const float *d_z, float *d_dzf, void *d_dzh,
                   tf_stream_t stream);
int tf_sg_pack(int ncell, int dof, int kp, const double *d_x, const double *d_t, const double *d_p,
               const float *sx, const float *st, const float *sp, float mu, float ds, void *d_x0,
               tf_stream_t stream);
int tf_sg_target(int ncell, int dof, const double *d_x0, const double *d_t, const double *d_x1, double ds,
                 const double *inv_scale, float *d_tgt, tf_stream_t stream);
int tf_sg_unpack(int ncell, int dof, int np, const float *d_out, const double *d_x0, const double *d_t,
                 double ds, const double *scale, double *d_xp, tf_stream_t stream);
int tf_sg_adam(int kp, int np, float *d_w, float *d_bias, const float *d_grad, float *d_m, float *d_v,
               float lr, float beta1, float beta2, float eps, int step, float grad_scale, void *d_wf,
               void *d_wb, tf_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* TFCUDA_H */
