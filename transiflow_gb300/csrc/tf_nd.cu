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

// Same panel factorisation with the (n - k) x nb panel staged in shared
// memory: pivot search, swaps and updates run on shared memory, the panel is
// written back once, and the recorded row swaps are then applied to the
// columns outside the panel.  Used whenever the panel fits (it does for every
// front of the 2D grids here; the kernel above is the fallback).
constexpr int PSTRIDE = NB + 1;

template <typename T>
__global__ void __launch_bounds__(THREADS) panel_smem_kernel(DevPlan P, int node0, int k, T *fronts, int32_t *piv,
                                                             int32_t *info) {
    extern __shared__ unsigned char smem_raw[];
    T *A = reinterpret_cast<T *>(smem_raw);     // [rows][PSTRIDE]
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    const int rows = n - k;
    T *F = fronts + P.front_off[node];
    int32_t *pv = piv + P.piv_off[node];
    __shared__ T sval[THREADS / 32];
    __shared__ int sidx[THREADS / 32];
    __shared__ int s_best;
    __shared__ int s_piv[NB];
    for (int t = threadIdx.x; t < rows * NB; t += THREADS) {
        const int r = t / NB, c = t % NB;
        A[r * PSTRIDE + c] = c < nb ? F[(size_t)(k + r) * f + k + c] : T(0);
    }
    __syncthreads();
    for (int lc = 0; lc < nb; ++lc) {
        T best = T(-1);
        int bi = lc;
        for (int r = lc + threadIdx.x; r < rows; r += THREADS) {
            T a = tabs(A[r * PSTRIDE + lc]);
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
            s_piv[lc] = i;
            pv[k + lc] = k + i;
            if (b == T(0) && info) atomicAdd(info, 1);
        }
        __syncthreads();
        const int r = s_best;
        if (r != lc && threadIdx.x < NB) {
            T t = A[lc * PSTRIDE + threadIdx.x];
            A[lc * PSTRIDE + threadIdx.x] = A[r * PSTRIDE + threadIdx.x];
            A[r * PSTRIDE + threadIdx.x] = t;
        }
        __syncthreads();
        T p = A[lc * PSTRIDE + lc];
        if (p == T(0)) p = T(1e-30);   // singular pivot: flagged through info
        const T rp = T(1) / p;
        for (int rr = lc + 1 + threadIdx.x; rr < rows; rr += THREADS) {
            T *row = A + rr * PSTRIDE;
            const T l = row[lc] * rp;
            row[lc] = l;
            for (int j = lc + 1; j < nb; ++j) row[j] -= l * A[lc * PSTRIDE + j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < rows * NB; t += THREADS) {
        const int r = t / NB, c = t % NB;
        if (c < nb) F[(size_t)(k + r) * f + k + c] = A[r * PSTRIDE + c];
    }
    // apply the swaps, in order, to the columns outside the panel
    for (int lc = 0; lc < nb; ++lc) {
        const int r = s_piv[lc];
        if (r != lc) {
            T *ra = F + (size_t)(k + lc) * f;
            T *rb = F + (size_t)(k + r) * f;
            for (int j = threadIdx.x; j < f - nb; j += THREADS) {
                const int col = j < k ? j : j + nb;
                T t = ra[col];
                ra[col] = rb[col];
                rb[col] = t;
            }
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

// Convert each front's pivot sequence (row c swapped with row piv[c], in
// order) into the permutation it composes to, in place: afterwards row c of
// the factored front corresponds to original own row piv[c].  Done once per
// factorisation so the solves gather in parallel.
__global__ void __launch_bounds__(256) pivots_to_permutation_kernel(DevPlan P, int nnodes, int32_t *piv) {
    extern __shared__ int sp[];
    const int node = blockIdx.x;
    if (node >= nnodes) return;
    const int n = P.n_own[node];
    int32_t *pv = piv + P.piv_off[node];
    int *perm = sp;
    int *seq = sp + n;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        perm[c] = c;
        seq[c] = pv[c];
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int c = 0; c < n; ++c) {
            const int r = seq[c];
            if (r != c) { int t = perm[c]; perm[c] = perm[r]; perm[r] = t; }
        }
    __syncthreads();
    for (int c = threadIdx.x; c < n; c += blockDim.x) pv[c] = perm[c];
}

// Forward sweep for the fronts of one height: permute, unit-lower solve,
// then subtract L21 y from the boundary unknowns.  Blocked by 32: warp 0
// solves the 32x32 diagonal block from shared memory, then every warp updates
// whole rows below it with coalesced row reads and a shuffle reduction.
constexpr int SB = 32;
constexpr int RPW = 8;   // rows per warp iteration in the sweep updates

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <typename T, int SOLVE_THREADS>
__global__ void __launch_bounds__(SOLVE_THREADS) fwd_kernel(DevPlan P, int node0, const T *fronts,
                                                            const int32_t *piv, double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *y = reinterpret_cast<T *>(smem_raw);
    __shared__ T D[SB][SB + 1];
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    const int32_t *pv = piv + P.piv_off[node];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = SOLVE_THREADS / 32;
    for (int c = threadIdx.x; c < n; c += SOLVE_THREADS) y[c] = (T)x[g[pv[c]]];
    __syncthreads();
    for (int k = 0; k < n; k += SB) {
        const int nb = min(SB, n - k);
        for (int t = threadIdx.x; t < nb * SB; t += SOLVE_THREADS) {
            const int r = t / SB, c = t % SB;
            D[r][c] = c < nb ? F[(size_t)(k + r) * f + k + c] : T(0);
        }
        __syncthreads();
        if (warp == 0) {
            T yi = lane < nb ? y[k + lane] : T(0);
            for (int c = 0; c < nb; ++c) {
                const T yc = __shfl_sync(0xffffffffu, yi, c);
                if (lane > c && lane < nb) yi -= D[lane][c] * yc;
            }
            if (lane < nb) y[k + lane] = yi;
        }
        __syncthreads();
        const T yk = lane < nb ? y[k + lane] : T(0);
        // 8 independent rows in flight per warp
        for (int r0 = k + nb + warp * RPW; r0 < n; r0 += nwarp * RPW) {
            T a[RPW];
#pragma unroll
            for (int q = 0; q < RPW; ++q) {
                const int r = r0 + q;
                a[q] = (lane < nb && r < n) ? F[(size_t)r * f + k + lane] * yk : T(0);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < RPW; ++q) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
            if (lane == 0)
#pragma unroll
                for (int q = 0; q < RPW; ++q)
                    if (r0 + q < n) y[r0 + q] -= a[q];
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += SOLVE_THREADS) x[g[c]] = (double)y[c];
    for (int r = n + warp; r < f; r += nwarp) {
        const T *row = F + (size_t)r * f;
        T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
        int c = lane;
        for (; c + 96 < n; c += 128) {
            s0 += row[c] * y[c];
            s1 += row[c + 32] * y[c + 32];
            s2 += row[c + 64] * y[c + 64];
            s3 += row[c + 96] * y[c + 96];
        }
        for (; c < n; c += 32) s0 += row[c] * y[c];
        const T s = warp_sum((s0 + s1) + (s2 + s3));
        if (lane == 0) atomicAdd(x + g[r], -(double)s);
    }
}

// Backward sweep: y = x_own - U12 x_bnd, then the blocked upper-triangular
// solve from the last block up.
template <typename T, int SOLVE_THREADS>
__global__ void __launch_bounds__(SOLVE_THREADS) bwd_kernel(DevPlan P, int node0, const T *fronts, double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *y = reinterpret_cast<T *>(smem_raw);
    __shared__ T D[SB][SB + 1];
    const int node = node0 + blockIdx.x;
    const int n = P.n_own[node], f = P.f[node];
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = SOLVE_THREADS / 32;
    // boundary values staged in shared memory (after y)
    T *xb = y + n;
    for (int b = threadIdx.x; b < f - n; b += SOLVE_THREADS) xb[b] = (T)x[g[n + b]];
    __syncthreads();
    for (int c = warp; c < n; c += nwarp) {
        const T *row = F + (size_t)c * f + n;
        const int nb_ = f - n;
        T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
        int b = lane;
        for (; b + 96 < nb_; b += 128) {
            s0 += row[b] * xb[b];
            s1 += row[b + 32] * xb[b + 32];
            s2 += row[b + 64] * xb[b + 64];
            s3 += row[b + 96] * xb[b + 96];
        }
        for (; b < nb_; b += 32) s0 += row[b] * xb[b];
        const T s = warp_sum((s0 + s1) + (s2 + s3));
        if (lane == 0) y[c] = (T)x[g[c]] - s;
    }
    __syncthreads();
    const int last = ((n - 1) / SB) * SB;
    for (int k = last; k >= 0; k -= SB) {
        const int nb = min(SB, n - k);
        for (int t = threadIdx.x; t < nb * SB; t += SOLVE_THREADS) {
            const int r = t / SB, c = t % SB;
            D[r][c] = c < nb ? F[(size_t)(k + r) * f + k + c] : T(0);
        }
        __syncthreads();
        if (warp == 0) {
            T yi = lane < nb ? y[k + lane] : T(0);
            for (int c = nb - 1; c >= 0; --c) {
                if (lane == c) yi = yi / D[c][c];
                const T yc = __shfl_sync(0xffffffffu, yi, c);
                if (lane < c) yi -= D[lane][c] * yc;
            }
            if (lane < nb) y[k + lane] = yi;
        }
        __syncthreads();
        const T yk = lane < nb ? y[k + lane] : T(0);
        for (int r0 = warp * RPW; r0 < k; r0 += nwarp * RPW) {
            T a[RPW];
#pragma unroll
            for (int q = 0; q < RPW; ++q) {
                const int r = r0 + q;
                a[q] = (lane < nb && r < k) ? F[(size_t)r * f + k + lane] * yk : T(0);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int q = 0; q < RPW; ++q) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
            if (lane == 0)
#pragma unroll
                for (int q = 0; q < RPW; ++q)
                    if (r0 + q < k) y[r0 + q] -= a[q];
        }
        __syncthreads();
    }
    for (int c = threadIdx.x; c < n; c += SOLVE_THREADS) x[g[c]] = (double)y[c];
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
static int panel_smem_limit() {
    static int limit = -1;
    if (limit < 0) {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        const int want = optin - 4096;   // leave room for the static shared arrays
        if (want > 0 && cudaFuncSetAttribute(panel_smem_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             want) == cudaSuccess)
            limit = want;
        else
            limit = 48 * 1024 - 4096;
        cudaGetLastError();
    }
    return limit;
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
            const size_t psm = sizeof(T) * (size_t)mo * PSTRIDE;
            if (psm <= (size_t)panel_smem_limit<T>()) {
                panel_smem_kernel<T><<<cnt, THREADS, psm, s>>>(D, node0, k, fronts, piv, info); launched();
            } else {
                panel_kernel<T><<<cnt, THREADS, 0, s>>>(D, node0, k, fronts, piv, info); launched();
            }
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
    int mo_all = 0;
    for (int h = 0; h < p->nlevels; ++h) mo_all = p->max_own[h] > mo_all ? p->max_own[h] : mo_all;
    pivots_to_permutation_kernel<<<p->nnodes, 256, 2 * sizeof(int) * (size_t)mo_all, s>>>(D, p->nnodes, piv);
    launched();
    return cuda_status();
}

template <typename T>
static int solve(const tf_nd_plan *p, const T *fronts, const int32_t *piv, double *x, cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!fronts || !piv || !x) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    // small fronts (the many leaves and low separators) get 128 threads, the
    // few large fronts near the root 512
    for (int h = 0; h < p->nlevels; ++h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const size_t sm = sizeof(T) * (size_t)p->max_own[h];
        if (p->max_own[h] > 256) {
            fwd_kernel<T, 512><<<cnt, 512, sm, s>>>(D, node0, fronts, piv, x); launched();
        } else {
            fwd_kernel<T, 128><<<cnt, 128, sm, s>>>(D, node0, fronts, piv, x); launched();
        }
    }
    for (int h = p->nlevels - 1; h >= 0; --h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const size_t sm = sizeof(T) * (size_t)p->max_f[h];
        if (p->max_own[h] > 256) {
            bwd_kernel<T, 512><<<cnt, 512, sm, s>>>(D, node0, fronts, x); launched();
        } else {
            bwd_kernel<T, 128><<<cnt, 128, sm, s>>>(D, node0, fronts, x); launched();
        }
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
