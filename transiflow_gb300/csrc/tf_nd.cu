// Nested-dissection multifrontal LU for the stencil Jacobian.
//
// The host plan (transiflow_gb300/ndplan.py) gives every elimination-tree
// node a dense frontal matrix F (f x f, row-major): its own unknowns first,
// then the boundary unknowns that ancestors eliminate.  Factorisation runs
// height by height (leaves first); all fronts of one height are processed by
// the same launches:
//   panel      pivoted LU of an NB-column panel over the own rows (one CTA per
//              front; pivots never leave the own rows),
//   lower      the boundary rows of the panel, X = F21 U11^-1,
//   urow       the panel's block row to the right, X = L11^-1 F12,
//   gemm       the trailing update F22 -= L21 U12 (64 x 64 tiles),
// after which the trailing block of each front is its Schur complement and is
// extend-added into the parent front.  The solves sweep the tree upwards
// (forward substitution, boundary updates) and downwards (back substitution).
// The reference this replaces is SuperLU via scipy.sparse.linalg.splu
// (transiflow/interface/SciPy.py:151, 194-202).

#include "tf_common.cuh"

namespace tf {
namespace nd {

constexpr int NB = 32;       // panel width
constexpr int TM = 64;       // gemm tile rows
constexpr int TN = 64;       // gemm tile cols
constexpr int THREADS = 256;

struct DevPlan {
    const int32_t *n_own, *f, *parent, *idx, *ea_map, *rank;
    const int64_t *front_off, *idx_off, *ea_off, *piv_off;
};

template <typename T>
__device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// Pivoted LU of columns [k, k+nb) over own rows [k, n), row swaps applied to
// the whole front row.  One CTA per front.
template <typename T>
__global__ void __launch_bounds__(THREADS) panel_kernel(DevPlan P, int node0, int k, T *fronts, int32_t *piv,
                                                        int32_t *info) {
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    T *F = fronts + P.front_off[node];
    int32_t *pv = piv + P.piv_off[node];
    __shared__ T sval[THREADS / 32];
    __shared__ int sidx[THREADS / 32];
    __shared__ int s_best;
    for (int c = k; c < k + nb; ++c) {
        // pivot search over own rows [c, n)
        T best = T(-1);
        int bi = c;
        for (int r = c + threadIdx.x; r < n; r += THREADS) {
            T a = tabs(F[(size_t)r * f + c]);
            if (a > best) { best = a; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            T ob = __shfl_down_sync(0xffffffffu, best, o);
            int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if ((threadIdx.x & 31) == 0) { sval[threadIdx.x >> 5] = best; sidx[threadIdx.x >> 5] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            T b = sval[0];
            int i = sidx[0];
            for (int w = 1; w < THREADS / 32; ++w)
                if (sval[w] > b || (sval[w] == b && sidx[w] < i)) { b = sval[w]; i = sidx[w]; }
            s_best = i;
            pv[c] = i;
            if (b == T(0) && info) atomicAdd(info, 1);
        }
        __syncthreads();
        const int r = s_best;
        if (r != c)
            for (int j = threadIdx.x; j < f; j += THREADS) {
                T t = F[(size_t)c * f + j];
                F[(size_t)c * f + j] = F[(size_t)r * f + j];
                F[(size_t)r * f + j] = t;
            }
        __syncthreads();
        T p = F[(size_t)c * f + c];
        if (p == T(0)) p = T(1e-30);   // singular pivot: flagged through info
        const T rp = T(1) / p;
        // scale and update the remaining panel columns over own rows below c
        for (int rr = c + 1 + threadIdx.x; rr < n; rr += THREADS) {
            T *row = F + (size_t)rr * f;
            const T l = row[c] * rp;
            row[c] = l;
            for (int j = c + 1; j < k + nb; ++j) row[j] -= l * F[(size_t)c * f + j];
        }
        __syncthreads();
    }
}

// Boundary rows [n, f) of the panel: X = F[r, k:k+nb] U_pp^-1
template <typename T>
__global__ void __launch_bounds__(THREADS) lower_kernel(DevPlan P, int node0, int k, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    T *F = fronts + P.front_off[node];
    __shared__ T U[NB][NB + 1];
    for (int t = threadIdx.x; t < nb * nb; t += THREADS) U[t / nb][t % nb] = F[(size_t)(k + t / nb) * f + k + t % nb];
    __syncthreads();
    const int r = n + blockIdx.x * THREADS + threadIdx.x;
    if (r >= f) return;
    T x[NB];
    T *row = F + (size_t)r * f + k;
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) x[c] = row[c];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        if (c < nb) {
            T s = x[c];
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (q < c) s -= x[q] * U[q][c];
            x[c] = s / U[c][c];
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) row[c] = x[c];
}

// Block row to the right of the panel: X = L_pp^-1 F[k:k+nb, j], j >= k+nb
template <typename T>
__global__ void __launch_bounds__(THREADS) urow_kernel(DevPlan P, int node0, int k, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    T *F = fronts + P.front_off[node];
    __shared__ T L[NB][NB + 1];
    for (int t = threadIdx.x; t < nb * nb; t += THREADS) L[t / nb][t % nb] = F[(size_t)(k + t / nb) * f + k + t % nb];
    __syncthreads();
    const int j = k + nb + blockIdx.x * THREADS + threadIdx.x;
    if (j >= f) return;
    T x[NB];
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) x[c] = F[(size_t)(k + c) * f + j];
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        if (c < nb) {
            T s = x[c];
#pragma unroll
            for (int q = 0; q < NB; ++q)
                if (q < c) s -= L[c][q] * x[q];
            x[c] = s;
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) F[(size_t)(k + c) * f + j] = x[c];
}

// Trailing update F[r][j] -= sum_q F[r][k+q] F[k+q][j], r, j >= k+nb
template <typename T>
__global__ void __launch_bounds__(THREADS) gemm_kernel(DevPlan P, int node0, int k, T *fronts) {
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    const int r0 = k + nb + blockIdx.y * TM, c0 = k + nb + blockIdx.x * TN;
    if (r0 >= f || c0 >= f) return;
    T *F = fronts + P.front_off[node];
    __shared__ T As[NB][TM + 1];   // As[q][r]
    __shared__ T Bs[NB][TN + 1];   // Bs[q][c]
    for (int t = threadIdx.x; t < NB * TM; t += THREADS) {
        const int q = t % NB, r = t / NB;
        As[q][r] = (q < nb && r0 + r < f) ? F[(size_t)(r0 + r) * f + k + q] : T(0);
    }
    for (int t = threadIdx.x; t < NB * TN; t += THREADS) {
        const int q = t / TN, c = t % TN;
        Bs[q][c] = (q < nb && c0 + c < f) ? F[(size_t)(k + q) * f + c0 + c] : T(0);
    }
    __syncthreads();
    const int tr = (threadIdx.x / 16) * 4, tc = (threadIdx.x % 16) * 4;
    T acc[4][4] = {};
#pragma unroll 8
    for (int q = 0; q < NB; ++q) {
        T a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { a[u] = As[q][tr + u]; b[u] = Bs[q][tc + u]; }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] += a[u] * b[v];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int r = r0 + tr + u;
        if (r >= f) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int c = c0 + tc + v;
            if (c < f) F[(size_t)r * f + c] -= acc[u][v];
        }
    }
}

// Scatter the (gauged) stencil-CSR values into the fronts.
template <typename T>
__global__ void scatter_kernel(int64_t m, const int64_t *__restrict__ pos, const int32_t *__restrict__ src,
                               const double *__restrict__ vals, T *fronts) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const double v = vals[src[e]];
    if (v != 0.0) atomicAdd(fronts + pos[e], (T)v);
}

// Extend-add of the Schur complements of fronts with child rank `rank` into
// their parents (one child of each parent per launch: no write conflicts).
template <typename T>
__global__ void extend_add_kernel(DevPlan P, int node0, int rank, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int par = P.parent[node];
    if (par < 0 || P.rank[node] != rank) return;
    const int n = P.n_own[node], f = P.f[node], b = f - n;
    const int fp = P.f[par];
    const T *F = fronts + P.front_off[node];
    T *G = fronts + P.front_off[par];
    const int32_t *m = P.ea_map + P.ea_off[node];
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)b * b;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int a = (int)(t / b), c = (int)(t % b);
        G[(size_t)m[a] * fp + m[c]] += F[(size_t)(n + a) * f + n + c];
    }
}

// Forward sweep for the fronts of one height: permute, unit-lower solve,
// then subtract L21 y from the boundary unknowns.
template <typename T>
__global__ void __launch_bounds__(THREADS) fwd_kernel(DevPlan P, int node0, const T *fronts, const int32_t *piv,
                                                      double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *y = reinterpret_cast<T *>(smem_raw);
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    const int32_t *pv = piv + P.piv_off[node];
    for (int c = threadIdx.x; c < n; c += THREADS) y[c] = (T)x[g[c]];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int c = 0; c < n; ++c) {
            const int r = pv[c];
            if (r != c) { T t = y[c]; y[c] = y[r]; y[r] = t; }
        }
    __syncthreads();
    for (int c = 0; c < n; ++c) {
        const T yc = y[c];
        for (int r = c + 1 + threadIdx.x; r < n; r += THREADS) y[r] -= F[(size_t)r * f + c] * yc;
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += THREADS) x[g[c]] = (double)y[c];
    for (int r = n + threadIdx.x; r < f; r += THREADS) {
        const T *row = F + (size_t)r * f;
        T s = T(0);
        for (int c = 0; c < n; ++c) s += row[c] * y[c];
        atomicAdd(x + g[r], -(double)s);
    }
}

// Backward sweep: y = x_own - U12 x_bnd, then upper-triangular solve.
template <typename T>
__global__ void __launch_bounds__(THREADS) bwd_kernel(DevPlan P, int node0, const T *fronts, double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *y = reinterpret_cast<T *>(smem_raw);
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    for (int c = threadIdx.x; c < n; c += THREADS) {
        const T *row = F + (size_t)c * f;
        T s = (T)x[g[c]];
        for (int b = n; b < f; ++b) s -= row[b] * (T)x[g[b]];
        y[c] = s;
    }
    __syncthreads();
    for (int c = n - 1; c >= 0; --c) {
        if (threadIdx.x == 0) y[c] = y[c] / F[(size_t)c * f + c];
        __syncthreads();
        const T yc = y[c];
        for (int r = threadIdx.x; r < c; r += THREADS) y[r] -= F[(size_t)r * f + c] * yc;
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += THREADS) x[g[c]] = (double)y[c];
}

static DevPlan dev_plan(const tf_nd_plan *p, const int32_t *rank) {
    DevPlan d;
    d.n_own = p->d_n_own;
    d.f = p->d_f;
    d.parent = p->d_parent;
    d.idx = p->d_idx;
    d.ea_map = p->d_ea_map;
    d.rank = rank;
    d.front_off = p->d_front_off;
    d.idx_off = p->d_idx_off;
    d.ea_off = p->d_ea_off;
    d.piv_off = p->d_piv_off;
    return d;
}

static int check_plan(const tf_nd_plan *p) {
    if (!p || p->n <= 0 || p->nnodes <= 0 || p->nlevels <= 0 || !p->level_ptr || !p->max_own || !p->max_f)
        return TF_ERR_ARG;
    if (!p->d_n_own || !p->d_f || !p->d_parent || !p->d_front_off || !p->d_idx_off || !p->d_idx ||
        !p->d_ea_off || !p->d_ea_map || !p->d_scat_pos || !p->d_scat_src || !p->d_piv_off || !p->d_rank)
        return TF_ERR_ARG;
    return TF_OK;
}

template <typename T>
static int factor(const tf_nd_plan *p, const double *vals, T *fronts, int32_t *piv, int32_t *info,
                  cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!vals || !fronts || !piv) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    if (cudaMemsetAsync(fronts, 0, sizeof(T) * (size_t)p->front_elems, s) != cudaSuccess) return TF_ERR_CUDA;
    launched();
    if (p->nscat > 0)
        scatter_kernel<T><<<(unsigned)((p->nscat + 255) / 256), 256, 0, s>>>(p->nscat, p->d_scat_pos, p->d_scat_src,
                                                                             vals, fronts); launched();
    for (int h = 0; h < p->nlevels; ++h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const int mo = p->max_own[h], mf = p->max_f[h];
        for (int k = 0; k < mo; k += NB) {
            panel_kernel<T><<<cnt, THREADS, 0, s>>>(D, node0, k, fronts, piv, info); launched();
            const int rest = mf - k - 1;
            if (mf > 0) {
                dim3 gl((mf + THREADS - 1) / THREADS, cnt);
                lower_kernel<T><<<gl, THREADS, 0, s>>>(D, node0, k, fronts); launched();
                urow_kernel<T><<<gl, THREADS, 0, s>>>(D, node0, k, fronts); launched();
            }
            if (rest > 0) {
                const int tiles = (rest + TM - 1) / TM;
                dim3 gg(tiles, tiles, cnt);
                gemm_kernel<T><<<gg, THREADS, 0, s>>>(D, node0, k, fronts); launched();
            }
        }
        for (int rank = 0; rank < 2; ++rank) {
            dim3 ge(64, cnt);
            extend_add_kernel<T><<<ge, 256, 0, s>>>(D, node0, rank, fronts); launched();
        }
    }
    return cuda_status();
}

template <typename T>
static int solve(const tf_nd_plan *p, const T *fronts, const int32_t *piv, double *x, cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!fronts || !piv || !x) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    for (int h = 0; h < p->nlevels; ++h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const size_t sm = sizeof(T) * (size_t)p->max_own[h];
        fwd_kernel<T><<<cnt, THREADS, sm, s>>>(D, node0, fronts, piv, x); launched();
    }
    for (int h = p->nlevels - 1; h >= 0; --h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const size_t sm = sizeof(T) * (size_t)p->max_own[h];
        bwd_kernel<T><<<cnt, THREADS, sm, s>>>(D, node0, fronts, x); launched();
    }
    return cuda_status();
}

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" int tf_nd_factor_f64(const tf_nd_plan *plan, const double *d_vals, double *d_fronts, int32_t *d_piv,
                                int32_t *d_info, tf_stream_t stream) {
    return nd::factor<double>(plan, d_vals, d_fronts, d_piv, d_info, (cudaStream_t)stream);
}

extern "C" int tf_nd_factor_f32(const tf_nd_plan *plan, const double *d_vals, float *d_fronts, int32_t *d_piv,
                                int32_t *d_info, tf_stream_t stream) {
    return nd::factor<float>(plan, d_vals, d_fronts, d_piv, d_info, (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv, double *d_x,
                               tf_stream_t stream) {
    return nd::solve<double>(plan, d_fronts, d_piv, d_x, (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv, double *d_x,
                               tf_stream_t stream) {
    return nd::solve<float>(plan, d_fronts, d_piv, d_x, (cudaStream_t)stream);
}
