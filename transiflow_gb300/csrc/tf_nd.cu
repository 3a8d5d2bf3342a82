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

#include <cooperative_groups.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

namespace tf {
namespace nd {

namespace cg = cooperative_groups;

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
// memory and its rows split over a cluster of CL CTAs (CL SMs: GB300 issues
// only two FP64 FMAs per SM and cycle, so one SM per panel is slow for the
// large fronts near the root).  Per column, with one cluster barrier: every
// CTA pushes its best row (value, index and the row itself) into every CTA's
// shared memory, and the owner of the diagonal row pushes that row too; after
// the barrier each CTA picks the same pivot from its local copies (largest
// magnitude, lowest row on ties), the two owners swap, and every CTA
// eliminates its own rows.  The exchange buffers alternate between columns.
// Afterwards each CTA writes its rows back and applies the recorded swaps, in
// order, to its share of the columns outside the panel.
constexpr int PSTRIDE = NB + 1;

template <typename T, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(THREADS)
    panel_cluster_kernel(DevPlan P, int node0, int k, T *fronts, int32_t *piv, int32_t *info) {
    extern __shared__ unsigned char smem_raw[];
    T *A = reinterpret_cast<T *>(smem_raw);     // [R][PSTRIDE]: panel rows [lo, hi)
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int node = node0 + blockIdx.x / CL;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;    // the same for every CTA of the cluster
    const int nb = min(NB, n - k);
    const int rows = n - k;
    const int R = (rows + CL - 1) / CL;
    const int lo = min(rows, q * R), hi = min(rows, lo + R);
    T *F = fronts + P.front_off[node];
    int32_t *pv = piv + P.piv_off[node];
    __shared__ T sval[THREADS / 32];
    __shared__ int sidx[THREADS / 32];
    __shared__ T cval[2][CL];
    __shared__ int cidx[2][CL];
    __shared__ T crow[2][CL][NB];
    __shared__ T lrow[2][NB];
    __shared__ int s_piv[NB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < (hi - lo) * NB; t += THREADS) {
        const int r = t / NB, c = t % NB;
        A[r * PSTRIDE + c] = c < nb ? F[(size_t)(k + lo + r) * f + k + c] : T(0);
    }
    __syncthreads();
    for (int lc = 0; lc < nb; ++lc) {
        const int par = lc & 1;
        T best = T(-1);
        int bi = 0x7fffffff;
        for (int r = max(lo, lc) + threadIdx.x; r < hi; r += THREADS) {
            const T a = tabs(A[(r - lo) * PSTRIDE + lc]);
            if (a > best) { best = a; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const T ob = __shfl_down_sync(0xffffffffu, best, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { sval[warp] = best; sidx[warp] = bi; }
        __syncthreads();
        const int ql = lc / R;
        if (warp == 0) {
            T b = sval[0];
            int i = sidx[0];
            for (int w = 1; w < THREADS / 32; ++w)
                if (sval[w] > b || (sval[w] == b && sidx[w] < i)) { b = sval[w]; i = sidx[w]; }
            const T v = (i < hi && lane < NB) ? A[(i - lo) * PSTRIDE + lane] : T(0);
            for (int d = 0; d < CL; ++d) {
                cluster.map_shared_rank(&crow[par][q][0], d)[lane] = v;
                if (lane == 0) {
                    *cluster.map_shared_rank(&cval[par][q], d) = b;
                    *cluster.map_shared_rank(&cidx[par][q], d) = i;
                }
            }
        } else if (warp == 1 && q == ql) {
            const T v = A[(lc - lo) * PSTRIDE + lane];
            for (int d = 0; d < CL; ++d) cluster.map_shared_rank(&lrow[par][0], d)[lane] = v;
        }
        cluster.sync();
        T b = T(-1);
        int r = 0x7fffffff, w = 0;
        for (int c = 0; c < CL; ++c)
            if (cval[par][c] > b || (cval[par][c] == b && cidx[par][c] < r)) { b = cval[par][c]; r = cidx[par][c]; w = c; }
        const T *prow = crow[par][w];
        if (r >= rows) { r = lc; b = T(0); prow = lrow[par]; }   // no comparable candidate (NaN column)
        if (threadIdx.x == 0) {
            s_piv[lc] = r;
            if (q == 0) {
                pv[k + lc] = k + r;
                if (b == T(0) && info) atomicAdd(info, 1);
            }
        }
        if (r != lc && threadIdx.x < NB) {
            if (q == ql) A[(lc - lo) * PSTRIDE + threadIdx.x] = prow[threadIdx.x];
            if (r >= lo && r < hi) A[(r - lo) * PSTRIDE + threadIdx.x] = lrow[par][threadIdx.x];
        }
        __syncthreads();
        T p = prow[lc];
        if (p == T(0)) p = T(1e-30);   // singular pivot: flagged through info
        const T rp = T(1) / p;
        for (int rr = max(lo, lc + 1) + threadIdx.x; rr < hi; rr += THREADS) {
            T *row = A + (rr - lo) * PSTRIDE;
            const T l = row[lc] * rp;
            row[lc] = l;
            for (int j = lc + 1; j < nb; ++j) row[j] -= l * prow[j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < (hi - lo) * NB; t += THREADS) {
        const int r = t / NB, c = t % NB;
        if (c < nb) F[(size_t)(k + lo + r) * f + k + c] = A[r * PSTRIDE + c];
    }
    // the swaps, in order, on this CTA's share of the columns outside the panel
    const int other = f - nb, C = (other + CL - 1) / CL;
    const int c0 = min(other, q * C), c1 = min(other, c0 + C);
    for (int j = c0 + threadIdx.x; j < c1; j += THREADS) {
        const int col = j < k ? j : j + nb;
        for (int lc = 0; lc < nb; ++lc) {
            const int r = s_piv[lc];
            if (r != lc) {
                T *ra = F + (size_t)(k + lc) * f + col;
                T *rb = F + (size_t)(k + r) * f + col;
                const T t = *ra;
                *ra = *rb;
                *rb = t;
            }
        }
    }
}

// Row swaps of a finished panel applied to this CTA's share [c0, c1) of the
// columns outside the panel (column j maps to j < k ? j : j + nb).  The
// swap sequence (row lc <-> row piv[lc], in order) only moves rows among
// S = [0, nb) and the distinct pivot rows >= nb, at most 2 nb rows; the
// composed permutation is worked out once, then the touched rows are
// gathered through shared memory 64 columns at a time, one round trip per
// chunk instead of nb dependent ones per column.  stage holds 2 NB x 64
// values; s_piv holds the pivot rows relative to k.
constexpr int SWAP_CHUNK = 64;

template <typename T>
__device__ void apply_panel_swaps(T *F, int f, int k, int nb, int c0, int c1, const int *s_piv, T *stage,
                                  int nthreads) {
    __shared__ int sl[2 * NB];     // touched rows (relative to k)
    __shared__ int pc[NB];         // compact slot of s_piv[t]
    __shared__ int srcc[2 * NB];   // slot whose old content ends in slot c
    __shared__ int nsl;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        const int p = lane < nb ? s_piv[lane] : -1;
        int first = lane;
        for (int t = 0; t < lane; ++t)
            if (s_piv[t] == p) { first = t; break; }
        const bool extra = p >= nb && first == lane;
        const unsigned ball = __ballot_sync(0xffffffffu, extra);
        if (lane < nb) sl[lane] = lane;
        if (extra) sl[nb + __popc(ball & ((1u << lane) - 1u))] = p;
        if (lane < nb) pc[lane] = p < nb ? p : nb + __popc(ball & ((1u << first) - 1u));
        if (lane == 0) nsl = nb + __popc(ball);
        __syncwarp();
        if (lane == 0) {
            int cur[2 * NB];
            const int m = nsl;
            for (int c = 0; c < m; ++c) cur[c] = c;
            for (int t = 0; t < nb; ++t) {
                const int a = t, b = pc[t];
                const int x = cur[a];
                cur[a] = cur[b];
                cur[b] = x;
            }
            for (int c = 0; c < m; ++c) srcc[c] = cur[c];
        }
    }
    __syncthreads();
    const int m = nsl;
    for (int j0 = c0; j0 < c1; j0 += SWAP_CHUNK) {
        const int w = min(SWAP_CHUNK, c1 - j0);
        for (int t = threadIdx.x; t < m * SWAP_CHUNK; t += nthreads) {
            const int c = t / SWAP_CHUNK, j = t % SWAP_CHUNK;
            if (j < w) {
                const int col = j0 + j < k ? j0 + j : j0 + j + nb;
                stage[c * SWAP_CHUNK + j] = F[(size_t)(k + sl[c]) * f + col];
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < m * SWAP_CHUNK; t += nthreads) {
            const int c = t / SWAP_CHUNK, j = t % SWAP_CHUNK;
            if (j < w && srcc[c] != c) {
                const int col = j0 + j < k ? j0 + j : j0 + j + nb;
                F[(size_t)(k + sl[c]) * f + col] = stage[srcc[c] * SWAP_CHUNK + j];
            }
        }
        __syncthreads();
    }
}

// Panel factorisation with every panel row held in the registers of one
// thread (PT threads, one row each, rows split over a cluster of CL CTAs).
// Per column: a warp all-reduce finds each warp's best row, whose lane parks
// the row in shared memory; warp 0 picks the CTA's best and pushes value,
// index and row into every CTA of the cluster (the holder of the diagonal
// row pushes that row too); after the one cluster barrier every thread picks
// the same pivot from its local copies, and the swap and the elimination
// happen in registers.  The exchange buffers alternate between columns,
// which makes the cluster barrier the only barrier per column.
template <typename T, int CL, int PT>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(PT)
    panel_reg_kernel(DevPlan P, int node0, int k, T *fronts, int32_t *piv, int32_t *info) {
    extern __shared__ unsigned char smem_raw[];
    T *stage = reinterpret_cast<T *>(smem_raw);   // [2 NB][SWAP_CHUNK] for the swaps
    constexpr int NW = PT / 32;
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int node = node0 + blockIdx.x / CL;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;    // the same for every CTA of the cluster
    const int nb = min(NB, n - k);
    const int rows = n - k;
    const int R = (rows + CL - 1) / CL;   // <= PT (host-checked)
    const int lo = min(rows, q * R), hi = min(rows, lo + R);
    T *F = fronts + P.front_off[node];
    int32_t *pv = piv + P.piv_off[node];
    __shared__ T wrow[NW][NB];
    __shared__ T wval[NW];
    __shared__ int widx[NW];
    __shared__ T lstage[NB];
    __shared__ T cval[2][CL];
    __shared__ T crcp[2][CL];      // 1 / (candidate's entry in column lc)
    __shared__ int cidx[2][CL];
    __shared__ T crow[2][CL][NB];
    __shared__ T lrow[2][NB];
    __shared__ int s_piv[NB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int my = lo + threadIdx.x;
    const bool have = my < hi;
    T a[NB];
    {
        const T *src = F + (size_t)(k + (have ? my : 0)) * f + k;
#pragma unroll
        for (int c = 0; c < NB; ++c) a[c] = (have && c < nb) ? src[c] : T(0);
    }
#pragma unroll
    for (int lc = 0; lc < NB; ++lc) {
        if (lc < nb) {
            const int par = lc & 1;
            const int ql = lc / R;
            T best = (have && my >= lc) ? tabs(a[lc]) : T(-1);
            int bi = (have && my >= lc) ? my : 0x7fffffff;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const T ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (have && bi == my) {
#pragma unroll
                for (int c = 0; c < NB; ++c) wrow[warp][c] = a[c];
            }
            if (lane == 0) { wval[warp] = best; widx[warp] = bi; }
            if (have && my == lc) {
#pragma unroll
                for (int c = 0; c < NB; ++c) lstage[c] = a[c];
            }
            __syncthreads();
            if (warp == 0) {
                T b = wval[0];
                int i = widx[0], ws = 0;
                for (int w = 1; w < NW; ++w)
                    if (wval[w] > b || (wval[w] == b && widx[w] < i)) { b = wval[w]; i = widx[w]; ws = w; }
                const T v = i < rows ? wrow[ws][lane] : T(0);
                T rcp = T(0);
                if (lane == lc) rcp = T(1) / (v == T(0) ? T(1e-30) : v);   // singular pivot: flagged through info
                for (int d = 0; d < CL; ++d) {
                    cluster.map_shared_rank(&crow[par][q][0], d)[lane] = v;
                    if (lane == 0) {
                        *cluster.map_shared_rank(&cval[par][q], d) = b;
                        *cluster.map_shared_rank(&cidx[par][q], d) = i;
                    }
                    if (lane == lc) *cluster.map_shared_rank(&crcp[par][q], d) = rcp;
                }
            } else if (warp == 1 && q == ql) {
                const T v = lstage[lane];
                for (int d = 0; d < CL; ++d) cluster.map_shared_rank(&lrow[par][0], d)[lane] = v;
            }
            cluster.sync();
            T b = T(-1);
            int r = 0x7fffffff, w = 0;
#pragma unroll
            for (int c = 0; c < CL; ++c)
                if (cval[par][c] > b || (cval[par][c] == b && cidx[par][c] < r)) { b = cval[par][c]; r = cidx[par][c]; w = c; }
            const T *prow = crow[par][w];
            T rp = crcp[par][w];
            if (r >= rows) {   // no comparable candidate (NaN column)
                r = lc;
                b = T(0);
                prow = lrow[par];
                rp = T(1) / prow[lc];
            }
            if (threadIdx.x == 0) {
                s_piv[lc] = r;
                if (q == 0) {
                    pv[k + lc] = k + r;
                    if (b == T(0) && info) atomicAdd(info, 1);
                }
            }
            if (have) {
                if (my == lc) {
#pragma unroll
                    for (int c = 0; c < NB; ++c) a[c] = prow[c];
                } else {
                    if (my == r) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) a[c] = lrow[par][c];
                    }
                    if (my > lc) {
                        const T l = a[lc] * rp;
                        a[lc] = l;
#pragma unroll
                        for (int j = lc + 1; j < NB; ++j) a[j] -= l * prow[j];
                    }
                }
            }
        }
    }
    if (have) {
        T *dst = F + (size_t)(k + my) * f + k;
#pragma unroll
        for (int c = 0; c < NB; ++c)
            if (c < nb) dst[c] = a[c];
    }
    __syncthreads();
    const int other = f - nb, C = (other + CL - 1) / CL;
    const int c0 = min(other, q * C), c1 = min(other, c0 + C);
    apply_panel_swaps(F, f, k, nb, c0, c1, s_piv, stage, PT);
}

// The two triangular solves with the panel's diagonal block run one row (or
// column) per thread in small CTAs, so that even a single large front spreads
// over many SMs; the diagonal of U is inverted once per CTA.
constexpr int TRSM_THREADS = 64;

// Boundary rows [n, f) of the panel: X = F[r, k:k+nb] U_pp^-1
template <typename T>
__global__ void __launch_bounds__(TRSM_THREADS) lower_kernel(DevPlan P, int node0, int k, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int r = n + blockIdx.x * TRSM_THREADS + threadIdx.x;
    if (n + blockIdx.x * TRSM_THREADS >= f) return;
    const int nb = min(NB, n - k);
    T *F = fronts + P.front_off[node];
    __shared__ T U[NB][NB + 1];
    __shared__ T rd[NB];
    for (int t = threadIdx.x; t < nb * nb; t += TRSM_THREADS) U[t / nb][t % nb] = F[(size_t)(k + t / nb) * f + k + t % nb];
    __syncthreads();
    if (threadIdx.x < nb) rd[threadIdx.x] = T(1) / U[threadIdx.x][threadIdx.x];
    __syncthreads();
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
            x[c] = s * rd[c];
        }
    }
#pragma unroll
    for (int c = 0; c < NB; ++c)
        if (c < nb) row[c] = x[c];
}

// Block row to the right of the panel: X = L_pp^-1 F[k:k+nb, j], j >= k+nb
template <typename T>
__global__ void __launch_bounds__(TRSM_THREADS) urow_kernel(DevPlan P, int node0, int k, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    if (k + nb + blockIdx.x * TRSM_THREADS >= f) return;
    T *F = fronts + P.front_off[node];
    __shared__ T L[NB][NB + 1];
    for (int t = threadIdx.x; t < nb * nb; t += TRSM_THREADS) L[t / nb][t % nb] = F[(size_t)(k + t / nb) * f + k + t % nb];
    __syncthreads();
    const int j = k + nb + blockIdx.x * TRSM_THREADS + threadIdx.x;
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

// ---------------------------------------------------------------------------
// Solve.  The factors are applied height by height with two launches per sweep
// and height: a triangular solve over each front's own rows and a
// matrix-vector product with the boundary coupling (L21 or U12) whose rows
// and columns are spread over many CTAs.  GB300 issues only two FP64 FMAs per
// SM and cycle, so no kernel here reduces across a warp with shuffles (the
// reduction would cost more FP64 issue slots than the products): a warp
// copies a 32 x 32 tile of the front into shared memory with cp.async
// (8- or 4-byte copies: rows of a front start at arbitrary alignment, which
// rules out TMA) and every lane forms the dot product of one row serially.
// The copies are issued ahead of the barrier or the tile before, so their
// latency overlaps other work.
constexpr int SB = 32;
constexpr int TSTRIDE = SB + 1;
constexpr int TILE = SB * TSTRIDE;      // elements of one padded 32 x 32 tile
constexpr int TRI_WARPS = 4;
constexpr int TRI_THREADS = 32 * TRI_WARPS;
constexpr int GEMV_WARPS = 2;
constexpr int GEMV_THREADS = 32 * GEMV_WARPS;
constexpr int GEMV_ROWS = 32 * GEMV_WARPS;
constexpr int GEMV_TILES = 4;           // column tiles per warp
constexpr int GEMV_COLS = GEMV_TILES * SB;

template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0)
                     : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
                     : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One warp: start copying the tile F[r0 .. r0+31][c0 .. c0+31] into buf
// (row-major, stride TSTRIDE) and commit it as one group; entries with row
// >= rmax or column >= cmax become zero.
template <typename T>
__device__ __forceinline__ void tile_issue(T *buf, const T *F, int f, int r0, int rmax, int c0, int cmax, int lane) {
    const bool colok = c0 + lane < cmax;
#pragma unroll 8
    for (int i = 0; i < SB; ++i) {
        const int r = r0 + i;
        const bool ok = colok && r < rmax;
        cp_async_elem(buf + i * TSTRIDE + lane, ok ? F + (size_t)r * f + c0 + lane : F, ok);
    }
    cp_async_commit();
}

// Lane l: sum_c buf[l][c] v[c].
template <typename T>
__device__ __forceinline__ T tile_dot(const T *buf, const T *v, int lane) {
    T s = T(0);
#pragma unroll 8
    for (int c = 0; c < SB; ++c) s += buf[lane * TSTRIDE + c] * v[c];
    return s;
}

// Triangular solves with the own block L11 (forward, unit lower, after the
// row permutation) or U11 (backward) of every front of one height.  A front's
// own rows form 32-row blocks; block b belongs to CTA b % CL of the front's
// cluster, which keeps the block's partial values in shared memory.  Block by
// block: the owner's warp 0 solves the diagonal block and pushes the 32
// solved values into every CTA of the cluster, then each CTA subtracts their
// contribution from its blocks further down (forward) or up (backward).
// Every warp commits exactly two cp.async groups per block step (its update
// tile, then the owner's next diagonal tile; either may be empty), so fixed
// wait_group counts select the right copies.
template <typename T, int CL, bool FWD>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(TRI_THREADS)
    tri_kernel(DevPlan P, int node0, const T *fronts, const int32_t *piv, double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *tiles = reinterpret_cast<T *>(smem_raw);        // [TRI_WARPS] update tiles
    T *dbuf = tiles + TRI_WARPS * TILE;                  // [2] diagonal tiles
    T *yl = dbuf + 2 * TILE;                             // [nloc][SB]
    __shared__ T ybuf[2][SB];
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int node = node0 + blockIdx.x / CL;
    const int n = P.n_own[node], f = P.f[node];
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nblk = (n + SB - 1) / SB;
    const int nloc = (nblk - q + CL - 1) / CL;
    T *mytile = tiles + warp * TILE;
    for (int t = threadIdx.x; t < nloc * SB; t += TRI_THREADS) {
        const int row = ((t / SB) * CL + q) * SB + t % SB;
        T v = T(0);
        if (row < n) v = FWD ? (T)x[g[piv[P.piv_off[node] + row]]] : (T)x[g[row]];
        yl[t] = v;
    }
    // the diagonal tile of this CTA's first block in solve order
    const int first_kb = FWD ? q : q + (nloc - 1) * CL;
    if (warp == 0 && nloc > 0)
        tile_issue(dbuf + ((first_kb / CL) & 1) * TILE, F, f, first_kb * SB, n, first_kb * SB, n, lane);
    __syncthreads();
    for (int step = 0; step < nblk; ++step) {
        const int kb = FWD ? step : nblk - 1 - step;
        const int k = kb * SB;
        // this warp's first block to update: below kb (forward) or above (backward)
        int lb, lend;
        if (FWD) {
            lb = (kb < q ? 0 : (kb - q) / CL + 1) + warp;
            lend = nloc;
        } else {
            lb = warp;
            lend = kb > q ? (kb - q + CL - 1) / CL : 0;
        }
        if (lb < lend)
            tile_issue(mytile, F, f, (lb * CL + q) * SB, n, k, n, lane);
        else
            cp_async_commit();
        const bool own = q == kb % CL && warp == 0;
        const int lbk = kb / CL;   // local index of kb when this CTA owns it
        const int next = FWD ? kb + CL : kb - CL;
        if (own && next >= 0 && next < nblk)
            tile_issue(dbuf + ((lbk + 1) & 1) * TILE, F, f, next * SB, n, next * SB, n, lane);
        else
            cp_async_commit();
        if (own) {
            cp_async_wait<2>();
            __syncwarp();
            const T *D = dbuf + (lbk & 1) * TILE;
            const int nb = min(SB, n - k);
            T *yb = yl + lbk * SB;
            T yi = yb[lane];
            if (FWD) {
                for (int c = 0; c < nb - 1; ++c) {
                    const T yc = __shfl_sync(0xffffffffu, yi, c);
                    if (lane > c) yi -= D[lane * TSTRIDE + c] * yc;
                }
            } else {
                const T rd = lane < nb ? T(1) / D[lane * TSTRIDE + lane] : T(0);
                for (int c = nb - 1; c >= 0; --c) {
                    if (lane == c) yi *= rd;
                    const T yc = __shfl_sync(0xffffffffu, yi, c);
                    if (lane < c) yi -= D[lane * TSTRIDE + c] * yc;
                }
            }
            yb[lane] = yi;
            for (int t = 0; t < CL; ++t) cluster.map_shared_rank(&ybuf[kb & 1][0], t)[lane] = yi;
        }
        cluster.sync();
        if (lb < lend) {
            const T *yk = ybuf[kb & 1];
            cp_async_wait<1>();
            __syncwarp();
            yl[lb * SB + lane] -= tile_dot(mytile, yk, lane);
            for (lb += TRI_WARPS; lb < lend; lb += TRI_WARPS) {
                __syncwarp();
                tile_issue(mytile, F, f, (lb * CL + q) * SB, n, k, n, lane);
                cp_async_wait<0>();
                __syncwarp();
                yl[lb * SB + lane] -= tile_dot(mytile, yk, lane);
            }
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    for (int t = threadIdx.x; t < nloc * SB; t += TRI_THREADS) {
        const int row = ((t / SB) * CL + q) * SB + t % SB;
        if (row < n) x[g[row]] = (double)yl[t];
    }
}

// Boundary couplings of every front of one height, one 32-row by 128-column
// piece per warp (grid: row pieces x fronts x column pieces), tiles double
// buffered:
//   forward  (FWD):  x[bnd] -= L21 y      rows [n, f), columns [0, n)
//   backward (!FWD): x[own] -= U12 x[bnd] rows [0, n), columns [n, f)
// Column pieces of one row (and, forward, sibling fronts sharing a boundary
// unknown) add into the same entry, hence the atomic update.
template <typename T, bool FWD>
__global__ void __launch_bounds__(GEMV_THREADS) bnd_kernel(DevPlan P, int node0, const T *fronts, double *x) {
    extern __shared__ unsigned char smem_raw[];
    T *tiles = reinterpret_cast<T *>(smem_raw);   // [GEMV_WARPS][2] tiles
    __shared__ T v[GEMV_COLS];
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int rlo = FWD ? n : 0, rhi = FWD ? f : n;
    const int clo = FWD ? 0 : n, chi = FWD ? n : f;
    const int rbase = rlo + blockIdx.x * GEMV_ROWS;
    const int cbase = clo + blockIdx.z * GEMV_COLS;
    if (rbase >= rhi || cbase >= chi) return;
    const int cend = min(chi, cbase + GEMV_COLS);
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = rbase + warp * SB;
    T *b0 = tiles + (2 * warp) * TILE, *b1 = b0 + TILE;
    if (r0 < rhi) tile_issue(b0, F, f, r0, rhi, cbase, chi, lane);
    for (int c = threadIdx.x; c < GEMV_COLS; c += GEMV_THREADS)
        v[c] = cbase + c < cend ? (T)x[g[cbase + c]] : T(0);
    __syncthreads();
    if (r0 >= rhi) return;
    T s = T(0);
    int t = 0;
    for (int c0 = cbase; c0 < cend; c0 += SB, ++t) {
        T *cur = (t & 1) ? b1 : b0;
        if (c0 + SB < cend) {
            tile_issue((t & 1) ? b0 : b1, F, f, r0, rhi, c0 + SB, chi, lane);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        s += tile_dot(cur, v + (c0 - cbase), lane);
        __syncwarp();
    }
    if (r0 + lane < rhi) atomicAdd(x + g[r0 + lane], -(double)s);
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

// Dynamic shared memory beyond a kernel's default limit (48 KiB minus its
// static shared memory) needs a per-kernel opt-in on the current device.
// Returns TF_ERR_SIZE when static plus dynamic shared memory would exceed
// what one CTA can have.
static int ensure_smem(const void *kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> allowed;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TF_ERR_CUDA;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(kernel, dev);
    const auto it = allowed.find(key);
    if (it != allowed.end() && it->second >= bytes) return TF_OK;
    cudaFuncAttributes a;
    int optin = 0;
    if (cudaFuncGetAttributes(&a, kernel) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return TF_ERR_CUDA;
    }
    if (bytes <= (size_t)a.maxDynamicSharedSizeBytes) {
        allowed[key] = (size_t)a.maxDynamicSharedSizeBytes;
        return TF_OK;
    }
    if (bytes + a.sharedSizeBytes > (size_t)optin) return TF_ERR_SIZE;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess) {
        cudaGetLastError();
        return TF_ERR_CUDA;
    }
    allowed[key] = bytes;
    return TF_OK;
}

// Panel launch over a cluster of CL CTAs per front.  Returns TF_ERR_SIZE when
// the per-CTA share of the panel does not fit in shared memory.
template <typename T, int CL>
static int launch_panel(const DevPlan &D, int node0, int cnt, int k, int rows, T *fronts, int32_t *piv,
                        int32_t *info, cudaStream_t s) {
    const size_t sm = sizeof(T) * (size_t)((rows + CL - 1) / CL) * PSTRIDE;
    const int e = ensure_smem((const void *)panel_cluster_kernel<T, CL>, sm);
    if (e) return e;
    panel_cluster_kernel<T, CL><<<cnt * CL, THREADS, sm, s>>>(D, node0, k, fronts, piv, info);
    launched();
    return TF_OK;
}

// Cluster size for cnt fronts with up to `rows` panel rows: about one CTA per
// SM in total and at least 32 rows per CTA.
static int panel_cluster_size(int cnt, int rows, int nsm) {
    int cl = 8;
    while (cl > 1 && (cnt * cl > nsm || rows < 32 * cl)) cl >>= 1;
    return cl;
}

template <typename T, int CL, int PT>
static int launch_panel_reg(const DevPlan &D, int node0, int cnt, int k, T *fronts, int32_t *piv, int32_t *info,
                            cudaStream_t s) {
    const size_t sm = sizeof(T) * 2 * NB * SWAP_CHUNK;
    const int e = ensure_smem((const void *)panel_reg_kernel<T, CL, PT>, sm);
    if (e) return e;
    panel_reg_kernel<T, CL, PT><<<cnt * CL, PT, sm, s>>>(D, node0, k, fronts, piv, info);
    launched();
    return TF_OK;
}

template <typename T, int CL>
static int launch_panel_reg_pt(const DevPlan &D, int node0, int cnt, int k, int rows, T *fronts, int32_t *piv,
                               int32_t *info, cudaStream_t s) {
    const int R = (rows + CL - 1) / CL;
    if (R <= 128) return launch_panel_reg<T, CL, 128>(D, node0, cnt, k, fronts, piv, info, s);
    if (R <= 256) return launch_panel_reg<T, CL, 256>(D, node0, cnt, k, fronts, piv, info, s);
    if (R <= 512) return launch_panel_reg<T, CL, 512>(D, node0, cnt, k, fronts, piv, info, s);
    return TF_ERR_SIZE;
}

template <typename T>
static int panel(const DevPlan &D, int node0, int cnt, int k, int rows, int nsm, T *fronts, int32_t *piv,
                 int32_t *info, cudaStream_t s) {
    // one register-held row per thread while a cluster of up to 8 CTAs
    // offers at most 512 rows per CTA
    for (int cl = panel_cluster_size(cnt, rows, nsm); cl <= 8; cl *= 2) {
        int e = TF_ERR_SIZE;
        switch (cl) {
        case 1: e = launch_panel_reg_pt<T, 1>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 2: e = launch_panel_reg_pt<T, 2>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 4: e = launch_panel_reg_pt<T, 4>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        default: e = launch_panel_reg_pt<T, 8>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        }
        if (e != TF_ERR_SIZE) return e;
    }
    // larger panels: rows staged in shared memory
    for (int cl = panel_cluster_size(cnt, rows, nsm); cl <= 8; cl *= 2) {
        int e = TF_ERR_SIZE;
        switch (cl) {
        case 1: e = launch_panel<T, 1>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 2: e = launch_panel<T, 2>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 4: e = launch_panel<T, 4>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        default: e = launch_panel<T, 8>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        }
        if (e != TF_ERR_SIZE) return e;
    }
    panel_kernel<T><<<cnt, THREADS, 0, s>>>(D, node0, k, fronts, piv, info);
    launched();
    return TF_OK;
}

template <typename T>
static int factor(const tf_nd_plan *p, const double *vals, T *fronts, int32_t *piv, int32_t *info,
                  cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!vals || !fronts || !piv) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    int mo_all = 0;
    for (int h = 0; h < p->nlevels; ++h) mo_all = p->max_own[h] > mo_all ? p->max_own[h] : mo_all;
    const size_t perm_smem = 2 * sizeof(int) * (size_t)mo_all;
    if ((e = ensure_smem((const void *)pivots_to_permutation_kernel, perm_smem))) return e;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return TF_ERR_CUDA;
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
            if ((e = panel<T>(D, node0, cnt, k, mo - k, nsm, fronts, piv, info, s))) return e;
            const int rest = mf - k - 1;
            if (mf > 0) {
                dim3 gl((mf + TRSM_THREADS - 1) / TRSM_THREADS, cnt);
                lower_kernel<T><<<gl, TRSM_THREADS, 0, s>>>(D, node0, k, fronts); launched();
                urow_kernel<T><<<gl, TRSM_THREADS, 0, s>>>(D, node0, k, fronts); launched();
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
    pivots_to_permutation_kernel<<<p->nnodes, 256, perm_smem, s>>>(D, p->nnodes, piv);
    launched();
    return cuda_status();
}

template <typename T, int CL, bool FWD>
static int launch_tri(const DevPlan &D, int node0, int cnt, int mo, const T *fronts, const int32_t *piv, double *x,
                      cudaStream_t s) {
    const int nblk = (mo + SB - 1) / SB;
    const size_t sm = sizeof(T) * ((size_t)(TRI_WARPS + 2) * TILE + (size_t)((nblk + CL - 1) / CL) * SB);
    const int e = ensure_smem((const void *)tri_kernel<T, CL, FWD>, sm);
    if (e) return e;
    tri_kernel<T, CL, FWD><<<cnt * CL, TRI_THREADS, sm, s>>>(D, node0, fronts, piv, x);
    launched();
    return TF_OK;
}

// Cluster size of a triangular-solve launch: about one CTA per SM in total
// and at least two row blocks per CTA.
template <typename T, bool FWD>
static int tri(const DevPlan &D, int node0, int cnt, int mo, int nsm, const T *fronts, const int32_t *piv,
               double *x, cudaStream_t s) {
    const int nblk = (mo + SB - 1) / SB;
    int cl = 8;
    while (cl > 1 && (cnt * cl > nsm || nblk < 2 * cl)) cl >>= 1;
    switch (cl) {
    case 8: return launch_tri<T, 8, FWD>(D, node0, cnt, mo, fronts, piv, x, s);
    case 4: return launch_tri<T, 4, FWD>(D, node0, cnt, mo, fronts, piv, x, s);
    case 2: return launch_tri<T, 2, FWD>(D, node0, cnt, mo, fronts, piv, x, s);
    default: return launch_tri<T, 1, FWD>(D, node0, cnt, mo, fronts, piv, x, s);
    }
}

template <typename T, bool FWD>
static void launch_bnd(const DevPlan &D, int node0, int cnt, int rows, int cols, const T *fronts, double *x,
                       cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return;
    dim3 grid((rows + GEMV_ROWS - 1) / GEMV_ROWS, cnt, (cols + GEMV_COLS - 1) / GEMV_COLS);
    bnd_kernel<T, FWD><<<grid, GEMV_THREADS, sizeof(T) * 2 * GEMV_WARPS * TILE, s>>>(D, node0, fronts, x);
    launched();
}

template <typename T>
static int solve(const tf_nd_plan *p, const T *fronts, const int32_t *piv, double *x, cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!fronts || !piv || !x) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return TF_ERR_CUDA;
    // rows and columns of the boundary products: at most max_f (boundary) and
    // max_own (own) per height
    for (int h = 0; h < p->nlevels; ++h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        const int mo = p->max_own[h], mf = p->max_f[h];
        if (cnt <= 0 || mo <= 0) continue;
        if ((e = tri<T, true>(D, node0, cnt, mo, nsm, fronts, piv, x, s))) return e;
        launch_bnd<T, true>(D, node0, cnt, mf, mo, fronts, x, s);
    }
    for (int h = p->nlevels - 1; h >= 0; --h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        const int mo = p->max_own[h], mf = p->max_f[h];
        if (cnt <= 0 || mo <= 0) continue;
        launch_bnd<T, false>(D, node0, cnt, mo, mf, fronts, x, s);
        if ((e = tri<T, false>(D, node0, cnt, mo, nsm, fronts, piv, x, s))) return e;
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
