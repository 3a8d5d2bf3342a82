// Sparse matrix and vector kernels: SpMV on the stencil CSR, the pressure
// gauge, export to the reference's compressed CSR, diagonal updates and the
// deterministic reductions used by GMRES and the continuation driver.

#include <mutex>

#include "tf_common.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// SpMV on the stencil CSR (rows hold 4..19 entries)
// ---------------------------------------------------------------------------
// SpMV with one lane per row: a warp takes 32 consecutive rows, stages their
// entries (contiguous in the CSR) in shared memory with coalesced loads, and
// every lane then sums its own row serially -- one FP64 FMA per entry and no
// shuffle sums.  (Eight lanes per row with a shuffle sum, the earlier
// design, spent more FP64 issue slots on the sums than on the products:
// GB300 issues two FP64 FMAs per SM and cycle.)
constexpr int SPR_WARPS = 4;
constexpr int SPR_CHUNK = 32 * 24;       // entries of a warp staged at once

template <typename TV>
__global__ void __launch_bounds__(32 * SPR_WARPS) spmv_rows_kernel(int n, const int32_t *__restrict__ rowptr,
                                                                   const int32_t *__restrict__ cols,
                                                                   const TV *__restrict__ vals,
                                                                   const double *__restrict__ x,
                                                                   double *__restrict__ y, double alpha,
                                                                   double beta) {
    __shared__ TV sv[SPR_WARPS][SPR_CHUNK];
    __shared__ int32_t sc[SPR_WARPS][SPR_CHUNK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = (blockIdx.x * SPR_WARPS + warp) * 32;
    if (r0 >= n) return;
    const int row = r0 + lane;
    const int base = __ldg(rowptr + r0), end = __ldg(rowptr + min(n, r0 + 32));
    const int b = row < n ? __ldg(rowptr + row) : end, e = row < n ? __ldg(rowptr + row + 1) : end;
    double acc = 0.0;
    for (int c0 = base; c0 < end; c0 += SPR_CHUNK) {
        const int c1 = min(end, c0 + SPR_CHUNK);
        for (int t = c0 + lane; t < c1; t += 32) {
            sv[warp][t - c0] = __ldg(vals + t);
            sc[warp][t - c0] = __ldg(cols + t);
        }
        __syncwarp();
        const int lo = max(b, c0), hi = min(e, c1);
        // unrolled so that several gathers of x are in flight per lane
#pragma unroll 4
        for (int t = lo; t < hi; ++t) acc += (double)sv[warp][t - c0] * __ldg(x + sc[warp][t - c0]);
        __syncwarp();
    }
    if (row < n) y[row] = beta == 0.0 ? alpha * acc : alpha * acc + beta * y[row];
}

// Copy with row g and column g replaced by a single -1 on the diagonal
// (SciPy.Interface.compute_bordered_matrix with fix_pressure_row, SciPy.py:93-103).
__global__ void gauge_kernel(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                             const double *__restrict__ vals, int g, double *__restrict__ out) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const int b = rowptr[row], e = rowptr[row + 1];
    bool placed = false;
    for (int t = b; t < e; ++t) {
        const int c = cols[t];
        double v = vals[t];
        if (row == g) {
            v = (c == g && !placed) ? -1.0 : 0.0;
            if (c == g) placed = true;
        } else if (c == g) {
            v = 0.0;
        }
        out[t] = v;
    }
}

__global__ void diag_axpy_kernel(int n, double a, const double *__restrict__ d, const double *__restrict__ x,
                                 double *__restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = y[i] + a * d[i] * x[i];
}

__global__ void add_diagonal_kernel(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                    double *__restrict__ vals, double a, const double *__restrict__ d) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    for (int t = rowptr[row]; t < rowptr[row + 1]; ++t)
        if (cols[t] == row) {
            vals[t] = vals[t] + a * d[row];
            return;
        }
}

// ---------------------------------------------------------------------------
// Export: CrsMatrix.compress on the stencil CSR (CrsMatrix.py:52-71).  Zero
// entries (dropped per entry by the assembly) are skipped, the rest sorted by
// column with a stable insertion sort, equal columns summed in stored order,
// and sums with |s| <= 1e-14 dropped.
// ---------------------------------------------------------------------------
constexpr int MAXROW = 64;
constexpr double DROP = 1e-14;

__device__ int compact_row(const int32_t *cols, const double *vals, int b, int e, int32_t *oc, double *ov) {
    int32_t c[MAXROW];
    double v[MAXROW];
    int m = 0;
    for (int t = b; t < e && m < MAXROW; ++t) {
        if (vals[t] == 0.0) continue;
        int32_t cc = cols[t];
        double vv = vals[t];
        int q = m++;
        while (q > 0 && c[q - 1] > cc) {
            c[q] = c[q - 1];
            v[q] = v[q - 1];
            --q;
        }
        c[q] = cc;
        v[q] = vv;
    }
    int out = 0;
    for (int q = 0; q < m;) {
        double s = 0.0;
        int r = q;
        while (r < m && c[r] == c[q]) s = s + v[r++];
        if (fabs(s) > DROP) {
            if (oc) {
                oc[out] = c[q];
                ov[out] = s;
            }
            ++out;
        }
        q = r;
    }
    return out;
}

__global__ void compact_count_kernel(int n, const int32_t *rowptr, const int32_t *cols, const double *vals,
                                     int32_t *count) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    count[row] = compact_row(cols, vals, rowptr[row], rowptr[row + 1], nullptr, nullptr);
}

__global__ void compact_write_kernel(int n, const int32_t *rowptr, const int32_t *cols, const double *vals,
                                     const int32_t *out_rowptr, int32_t *out_cols, double *out_vals) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const int o = out_rowptr[row];
    compact_row(cols, vals, rowptr[row], rowptr[row + 1], out_cols + o, out_vals + o);
}

// Exclusive scan of n+1 int32 values in place (last input ignored): block
// scans of 4096 elements, a single-block scan of the block totals, then a
// fix-up pass.
constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = SCAN_BLOCK * SCAN_ITEMS;

__device__ int block_exclusive_scan(int x, int *tmp, int *total) {
    const int tid = threadIdx.x;
    tmp[tid] = x;
    __syncthreads();
    for (int off = 1; off < SCAN_BLOCK; off <<= 1) {
        int y = tid >= off ? tmp[tid - off] : 0;
        __syncthreads();
        tmp[tid] += y;
        __syncthreads();
    }
    int incl = tmp[tid];
    if (total) *total = tmp[SCAN_BLOCK - 1];
    __syncthreads();
    return incl - x;
}

__global__ void scan_blocks_kernel(int n, int32_t *a, int32_t *block_tot) {
    __shared__ int tmp[SCAN_BLOCK];
    __shared__ int tot;
    const int base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
    for (int q = 0; q < SCAN_ITEMS; ++q) {
        v[q] = base + q < n ? a[base + q] : 0;
        s += v[q];
    }
    int ex = block_exclusive_scan(s, tmp, &tot);
    for (int q = 0; q < SCAN_ITEMS; ++q) {
        if (base + q < n) a[base + q] = ex;
        ex += v[q];
    }
    if (threadIdx.x == 0) block_tot[blockIdx.x] = tot;
}

__global__ void scan_totals_kernel(int nb, int32_t *block_tot, int32_t *a, int n) {
    __shared__ int tmp[SCAN_BLOCK];
    __shared__ int tot;
    int x = threadIdx.x < nb ? block_tot[threadIdx.x] : 0;
    int ex = block_exclusive_scan(x, tmp, &tot);
    if (threadIdx.x < nb) block_tot[threadIdx.x] = ex;
    if (threadIdx.x == 0) a[n] = tot;
}

__global__ void scan_fixup_kernel(int n, int32_t *a, const int32_t *block_tot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += block_tot[i / SCAN_CHUNK];
}

// ---------------------------------------------------------------------------
// Reductions and vector updates
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 304;   // 2 x 152 SMs

// partial[b*k + j] = sum over the block's grid-stride chunk of V_j . w.
// The vectors are taken MD_KV at a time, so w is read once per group of
// MD_KV vectors (not once per vector); every dot product still adds its
// terms in the same order, so the result does not depend on the grouping.
constexpr int MD_KV = 8;

__global__ void __launch_bounds__(RED_THREADS) mdot_partial_kernel(int n, int k, const double *__restrict__ V,
                                                                   long long ldv, const double *__restrict__ w,
                                                                   double *__restrict__ partial) {
    __shared__ double red[RED_THREADS / 32][MD_KV];
    for (int j0 = 0; j0 < k; j0 += MD_KV) {
        const int kv = min(MD_KV, k - j0);
        double acc[MD_KV];
#pragma unroll
        for (int q = 0; q < MD_KV; ++q) acc[q] = 0.0;
        const double *v = V + (long long)j0 * ldv;
        for (int i = blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += gridDim.x * RED_THREADS) {
            const double wi = __ldg(w + i);
#pragma unroll
            for (int q = 0; q < MD_KV; ++q)
                if (q < kv) acc[q] += __ldg(v + (long long)q * ldv + i) * wi;
        }
#pragma unroll
        for (int q = 0; q < MD_KV; ++q) {
            double a = acc[q];
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][q] = a;
        }
        __syncthreads();
        if (threadIdx.x < kv) {
            double sum = 0.0;
            for (int r = 0; r < RED_THREADS / 32; ++r) sum += red[r][threadIdx.x];
            partial[blockIdx.x * k + j0 + threadIdx.x] = sum;
        }
        __syncthreads();
    }
}

__global__ void mdot_final_kernel(int nb, int k, const double *__restrict__ partial, double *__restrict__ out) {
    const int j = blockIdx.x;
    __shared__ double red[32];
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += partial[b * k + j];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x / 32); ++q) s += red[q];
        out[j] = s;
    }
}

__global__ void mgs_update_kernel(int n, int k, const double *__restrict__ V, long long ldv,
                                  const double *__restrict__ h, double *__restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc = w[i];
    for (int j = 0; j < k; ++j) acc -= __ldg(V + (long long)j * ldv + i) * __ldg(h + j);
    w[i] = acc;
}

__global__ void axpby_kernel(int n, double a, const double *x, double b, const double *y, double *z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = x ? a * x[i] : 0.0;
    z[i] = y ? xi + b * y[i] : xi;
}

__global__ void div_kernel(int n, const double *x, double s, double *z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = x[i] / s;
}

// z *= 1 / sqrt(*nrm2), the square norm read on the device (a zero norm
// makes z non-finite: a breakdown the caller detects).
__global__ void scale_rsqrt_kernel(int n, const double *nrm2, double *z) {
    const double r = rsqrt(*nrm2);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] *= r;
}

__global__ void fill_kernel(int n, double a, double *z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = a;
}

__global__ void cast_kernel(int n, const double *x, float *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (float)x[i];
}

}  // namespace tf

using namespace tf;

std::atomic<long long> tf::g_launches{0};

extern "C" long long tf_launch_count(void) { return g_launches.load(); }
extern "C" void tf_launch_count_reset(void) { g_launches.store(0); }

// A stream of its own for one caller (one solver instance, one helper
// stream): non-blocking with respect to the legacy default stream, and never
// shared, unlike pooled streams, so a graph capture on it cannot meet another
// thread's work.
extern "C" int tf_stream_create(tf_stream_t *out) {
    if (!out) return TF_ERR_ARG;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TF_ERR_CUDA;
    *out = (tf_stream_t)s;
    return TF_OK;
}

extern "C" int tf_stream_destroy(tf_stream_t stream) {
    if (!stream) return TF_ERR_ARG;
    return cudaStreamDestroy((cudaStream_t)stream) == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

static inline int blocks_for(long long n, int t) { return (int)((n + t - 1) / t); }

extern "C" int tf_gauge_values(int n, const int32_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                               int gauge, double *d_out, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_out || gauge < 0 || gauge >= n) return TF_ERR_ARG;
    gauge_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_rowptr, d_cols, d_vals, gauge, d_out); launched();
    return cuda_status();
}

extern "C" int tf_spmv_f64(int n, const int32_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                           const double *d_x, double *d_y, double alpha, double beta, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_x || !d_y) return TF_ERR_ARG;
    spmv_rows_kernel<double><<<blocks_for((long long)n, 32 * SPR_WARPS), 32 * SPR_WARPS, 0, (cudaStream_t)stream>>>(
        n, d_rowptr, d_cols, d_vals, d_x, d_y, alpha, beta); launched();
    return cuda_status();
}

extern "C" int tf_spmv_f32(int n, const int32_t *d_rowptr, const int32_t *d_cols, const float *d_vals,
                           const double *d_x, double *d_y, double alpha, double beta, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_x || !d_y) return TF_ERR_ARG;
    spmv_rows_kernel<float><<<blocks_for((long long)n, 32 * SPR_WARPS), 32 * SPR_WARPS, 0, (cudaStream_t)stream>>>(
        n, d_rowptr, d_cols, d_vals, d_x, d_y, alpha, beta); launched();
    return cuda_status();
}

// ---------------------------------------------------------------------------
// Equilibration of an operator before a low-precision factorisation: row
// scales d_r = 2^-e (max_j |a_ij| = f 2^e, 1/2 <= f < 1), then column scales
// d_c of the row-scaled matrix the same way, and the scaled values
// d_r[i] a_ij d_c[j].  Powers of two: the scaling itself is exact in FP64.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pow2_recip(double m) {
    int e = 0;
    frexp(m, &e);
    return ldexp(1.0, -e);
}

__global__ void eq_rows_kernel(int n, const int32_t *__restrict__ rowptr, const double *__restrict__ vals,
                               double *__restrict__ dr, unsigned long long *__restrict__ cbits) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double m = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) m = fmax(m, fabs(vals[k]));
    dr[r] = m > 0.0 ? pow2_recip(m) : 1.0;
    cbits[r] = 0ull;
}

// column maxima of the row-scaled values: non-negative doubles order like
// their bit patterns, so an integer atomicMax on the bits is a maximum
__global__ void eq_cols_kernel(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                               const double *__restrict__ vals, const double *__restrict__ dr,
                               unsigned long long *__restrict__ cbits) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double s = dr[r];
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
        const double a = fabs(vals[k] * s);
        if (a > 0.0) atomicMax(cbits + cols[k], (unsigned long long)__double_as_longlong(a));
    }
}

__global__ void eq_finish_kernel(int n, unsigned long long *__restrict__ cbits) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const double m = __longlong_as_double((long long)cbits[j]);
    reinterpret_cast<double *>(cbits)[j] = m > 0.0 ? pow2_recip(m) : 1.0;
}

__global__ void eq_scale_kernel(int n, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                                const double *vals, const double *__restrict__ dr, const double *__restrict__ dc,
                                double *out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double s = dr[r];
    for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) out[k] = vals[k] * s * dc[cols[k]];
}

__global__ void vec_mul_kernel(int n, const double *__restrict__ d, const double *x, double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = d[i] * x[i];
}

extern "C" int tf_equilibrate(int n, const int32_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                              double *d_rscale, double *d_cscale, double *d_out, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_rscale || !d_cscale || !d_out) return TF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    auto *cbits = reinterpret_cast<unsigned long long *>(d_cscale);
    const int b = blocks_for(n, 256);
    eq_rows_kernel<<<b, 256, 0, s>>>(n, d_rowptr, d_vals, d_rscale, cbits);
    eq_cols_kernel<<<b, 256, 0, s>>>(n, d_rowptr, d_cols, d_vals, d_rscale, cbits);
    eq_finish_kernel<<<b, 256, 0, s>>>(n, cbits);
    eq_scale_kernel<<<b, 256, 0, s>>>(n, d_rowptr, d_cols, d_vals, d_rscale, d_cscale, d_out);
    launched(4);
    return cuda_status();
}

extern "C" int tf_vec_mul(int n, const double *d_d, const double *d_x, double *d_y, tf_stream_t stream) {
    if (n <= 0 || !d_d || !d_x || !d_y) return TF_ERR_ARG;
    vec_mul_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_d, d_x, d_y);
    launched();
    return cuda_status();
}

extern "C" int tf_diag_axpy(int n, double a, const double *d_diag, const double *d_x, double *d_y,
                            tf_stream_t stream) {
    if (n <= 0 || !d_diag || !d_x || !d_y) return TF_ERR_ARG;
    diag_axpy_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, a, d_diag, d_x, d_y); launched();
    return cuda_status();
}

extern "C" int tf_add_diagonal(int n, const int32_t *d_rowptr, const int32_t *d_cols, double *d_vals, double a,
                               const double *d_diag, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_diag) return TF_ERR_ARG;
    add_diagonal_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_rowptr, d_cols, d_vals, a,
                                                                              d_diag); launched();
    return cuda_status();
}

extern "C" size_t tf_csr_compact_workspace_bytes(int n) {
    return sizeof(int32_t) * (size_t)(blocks_for((long long)n + 1, SCAN_CHUNK) + 1);
}

extern "C" int tf_csr_compact(int n, const int32_t *d_rowptr, const int32_t *d_cols, const double *d_vals,
                              int32_t *d_out_rowptr, int32_t *d_out_cols, double *d_out_vals, int64_t *nnz,
                              void *d_work, size_t work_bytes, tf_stream_t stream) {
    if (n <= 0 || !d_rowptr || !d_cols || !d_vals || !d_out_rowptr) return TF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = blocks_for((long long)n, SCAN_CHUNK);
    if (nb > SCAN_BLOCK) return TF_ERR_SIZE;
    if (!d_work || work_bytes < tf_csr_compact_workspace_bytes(n)) return TF_ERR_ARG;
    int32_t *tot = (int32_t *)d_work;
    if (!d_out_cols) {
        compact_count_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n, d_rowptr, d_cols, d_vals, d_out_rowptr); launched();
        scan_blocks_kernel<<<nb, SCAN_BLOCK, 0, s>>>(n, d_out_rowptr, tot); launched();
        scan_totals_kernel<<<1, SCAN_BLOCK, 0, s>>>(nb, tot, d_out_rowptr, n); launched();
        scan_fixup_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, d_out_rowptr, tot); launched();
        if (nnz) {
            int32_t h = 0;
            if (cudaMemcpyAsync(&h, d_out_rowptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
                return TF_ERR_CUDA;
            if (cudaStreamSynchronize(s) != cudaSuccess) return TF_ERR_CUDA;
            *nnz = h;
        }
        return cuda_status();
    }
    if (!d_out_vals) return TF_ERR_ARG;
    compact_write_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n, d_rowptr, d_cols, d_vals, d_out_rowptr, d_out_cols,
                                                          d_out_vals); launched();
    return cuda_status();
}

extern "C" size_t tf_vec_mdot_workspace_bytes(int n, int k) {
    (void)n;
    return sizeof(double) * (size_t)RED_BLOCKS * (size_t)(k > 0 ? k : 1);
}

extern "C" int tf_vec_mdot(int n, int k, const double *d_V, long long ldv, const double *d_w, double *d_out,
                           void *d_work, size_t work_bytes, tf_stream_t stream) {
    if (n <= 0 || k <= 0 || k > 256 || !d_V || !d_w || !d_out || ldv < n) return TF_ERR_ARG;
    if (!d_work || work_bytes < tf_vec_mdot_workspace_bytes(n, k)) return TF_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int nb = blocks_for(n, RED_THREADS);
    if (nb > RED_BLOCKS) nb = RED_BLOCKS;
    mdot_partial_kernel<<<nb, RED_THREADS, 0, s>>>(n, k, d_V, ldv, d_w, (double *)d_work); launched();
    mdot_final_kernel<<<k, 128, 0, s>>>(nb, k, (const double *)d_work, d_out); launched();
    return cuda_status();
}

extern "C" int tf_vec_mgs_update(int n, int k, const double *d_V, long long ldv, const double *d_h, double *d_w,
                                 tf_stream_t stream) {
    if (n <= 0 || k <= 0 || k > 256 || !d_V || !d_h || !d_w || ldv < n) return TF_ERR_ARG;
    mgs_update_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, k, d_V, ldv, d_h, d_w); launched();
    return cuda_status();
}

// ---------------------------------------------------------------------------
// Multi-dot without caller-provided or allocated scratch.
//
// Some callers cannot allocate device memory at the point where they need an
// inner product: a host application that hands this library a fixed device
// memory budget up front and forbids any further cudaMalloc, or a solver loop
// that must not pay the implicit device-wide synchronisation cudaMalloc and
// cudaFree can cause.  tf_vec_mdot_noalloc gives them the same reduction as
// tf_vec_mdot with its per-block partial sums kept in a fixed array that every
// GPU loading this library holds until the process exits.
//
// Limit: k <= TF_MDOT_NOALLOC_MAX_K vectors (the array holds RED_BLOCKS x
// TF_MDOT_NOALLOC_MAX_K doubles, 152 KiB).  All calls share the array, so
// calls that overlap on the GPU (different streams without ordering between
// them) race and must not be issued.  Each call writes every partial sum it
// later reads, so nothing has to be cleared between calls.
// ---------------------------------------------------------------------------
#define TF_MDOT_NOALLOC_MAX_K 64

static __device__ __align__(256) double g_mdot_noalloc_scratch[RED_BLOCKS * TF_MDOT_NOALLOC_MAX_K];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {};
}  // namespace

// Device address of the scratch array for the current device.  The host
// symbol g_mdot_noalloc_scratch is only a stand-in for the array, not a
// device address, so the address is looked up once per device with that
// device current and cached for the life of the process (a cudaDeviceReset
// of that device invalidates it; the header says so).
static int noalloc_scratch(double **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TF_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return TF_ERR_SIZE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_mdot_noalloc_scratch) != cudaSuccess || !p) return TF_ERR_CUDA;
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return TF_OK;
}

extern "C" int tf_vec_mdot_noalloc(int n, int k, const double *d_V, long long ldv, const double *d_w,
                                   double *d_out, tf_stream_t stream) {
    if (n <= 0 || k <= 0 || !d_V || !d_w || !d_out || ldv < n) return TF_ERR_ARG;
    if (k > TF_MDOT_NOALLOC_MAX_K) return TF_ERR_SIZE;
    double *scratch = nullptr;
    int e = noalloc_scratch(&scratch);
    if (e) return e;
    cudaStream_t s = (cudaStream_t)stream;
    int nb = blocks_for(n, RED_THREADS);
    if (nb > RED_BLOCKS) nb = RED_BLOCKS;
    mdot_partial_kernel<<<nb, RED_THREADS, 0, s>>>(n, k, d_V, ldv, d_w, scratch); launched();
    mdot_final_kernel<<<k, 128, 0, s>>>(nb, k, (const double *)scratch, d_out); launched();
    return cuda_status();
}

/* z = a x + b y; x or y may be NULL (treated as absent); z may alias x or y. */
extern "C" int tf_vec_axpby(int n, double a, const double *d_x, double b, const double *d_y, double *d_z,
                            tf_stream_t stream) {
    if (n <= 0 || !d_z) return TF_ERR_ARG;
    axpby_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, a, d_x, b, d_y, d_z); launched();
    return cuda_status();
}

/* z = x / s with IEEE division per element (z may alias x).                */
extern "C" int tf_vec_div(int n, const double *d_x, double s, double *d_z, tf_stream_t stream) {
    if (n <= 0 || !d_x || !d_z) return TF_ERR_ARG;
    div_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_x, s, d_z); launched();
    return cuda_status();
}

extern "C" int tf_vec_scale_rsqrt(int n, const double *d_nrm2, double *d_z, tf_stream_t stream) {
    if (n <= 0 || !d_nrm2 || !d_z) return TF_ERR_ARG;
    scale_rsqrt_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_nrm2, d_z);
    launched();
    return cuda_status();
}

extern "C" int tf_vec_fill(int n, double a, double *d_z, tf_stream_t stream) {
    if (n <= 0 || !d_z) return TF_ERR_ARG;
    fill_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, a, d_z); launched();
    return cuda_status();
}

extern "C" int tf_vec_to_f32(int n, const double *d_x, float *d_y, tf_stream_t stream) {
    if (n <= 0 || !d_x || !d_y) return TF_ERR_ARG;
    cast_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_x, d_y); launched();
    return cuda_status();
}
