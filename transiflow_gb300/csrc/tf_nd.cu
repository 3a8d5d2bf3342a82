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

#include "tf_nd.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

namespace tf {
namespace nd {

// The two triangular solves with the panel's diagonal block run one row (or
// column) per thread in small CTAs, so that even a single large front spreads
// over many SMs; the diagonal of U is inverted once per CTA.
constexpr int TRSM_THREADS = 64;

// Boundary rows [n, f) of the panel: X = F[r, k:k+nb] U_pp^-1
template <typename T>
__device__ __forceinline__ void lower_rows(const DevPlan &P, int node0, int k, T *fronts) {
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

// Block row to the right of the panel: X = L_pp^-1 F[k:k+nb, j] for the
// columns j of the update region `mode` (UPD_ALL: [k+nb, f); UPD_COLS: the
// outer block's columns [k+nb, E); UPD_ROWS: the columns [E, f) right of it)
template <typename T>
__device__ __forceinline__ void urow_cols(const DevPlan &P, int node0, int k, int K0, int mode, T *fronts) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    int jlo = k + nb, jhi = f;
    if (mode != UPD_ALL) {
        const int E = min(K0 + KB, n);
        if (mode == UPD_COLS) jhi = E;
        else jlo = E;
    }
    if (jlo + blockIdx.x * TRSM_THREADS >= jhi) return;
    T *F = fronts + P.front_off[node];
    __shared__ T L[NB][NB + 1];
    for (int t = threadIdx.x; t < nb * nb; t += TRSM_THREADS) L[t / nb][t % nb] = F[(size_t)(k + t / nb) * f + k + t % nb];
    __syncthreads();
    const int j = jlo + blockIdx.x * TRSM_THREADS + threadIdx.x;
    if (j >= jhi) return;
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

// Both triangular solves of one panel step in one launch (grid.z + zbase =
// 0: the boundary rows, 1: the block row over the columns of `mode`); they
// are independent of each other.
template <typename T>
__global__ void __launch_bounds__(TRSM_THREADS) trsm_kernel(DevPlan P, int node0, int k, int K0, int mode, int zbase,
                                                            T *fronts) {
    if (blockIdx.z + zbase == 0) lower_rows(P, node0, k, fronts);
    else urow_cols(P, node0, k, K0, mode, fronts);
}

// Rows [rlo, rhi) and columns [clo, chi) of the trailing update of the
// panel at column k (see UPD_*).
struct Region {
    int rlo, rhi, clo, chi;
};
__device__ __forceinline__ Region update_region(int mode, int k, int nb, int K0, int n, int f) {
    Region g{k + nb, f, k + nb, f};
    if (mode != UPD_ALL) {
        const int E = min(K0 + KB, n);
        if (mode == UPD_COLS) {
            g.chi = E;
        } else {
            g.rhi = E;
            g.clo = E;
        }
    }
    return g;
}

// Trailing update F[r][j] -= sum_q F[r][k+q] F[k+q][j] over one region
template <typename T>
__global__ void __launch_bounds__(THREADS) gemm_kernel(DevPlan P, int node0, int k, int K0, int mode, T *fronts) {
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    const Region g = update_region(mode, k, nb, K0, n, f);
    const int r0 = g.rlo + blockIdx.y * TM, c0 = g.clo + blockIdx.x * TN;
    if (r0 >= g.rhi || c0 >= g.chi) return;
    T *F = fronts + P.front_off[node];
    __shared__ T As[NB][TM + 1];   // As[q][r]
    __shared__ T Bs[NB][TN + 1];   // Bs[q][c]
    for (int t = threadIdx.x; t < NB * TM; t += THREADS) {
        const int q = t % NB, r = t / NB;
        As[q][r] = (q < nb && r0 + r < g.rhi) ? F[(size_t)(r0 + r) * f + k + q] : T(0);
    }
    for (int t = threadIdx.x; t < NB * TN; t += THREADS) {
        const int q = t / TN, c = t % TN;
        Bs[q][c] = (q < nb && c0 + c < g.chi) ? F[(size_t)(k + q) * f + c0 + c] : T(0);
    }
    __syncthreads();
    // warp w owns rows [16 (w / 2), +16) and columns [32 (w % 2), +32) of the
    // tile; a warp entirely past the front's edge skips its products (the FP64
    // pipe is the bound, and the last tiles of a front are often partial)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wr = (warp >> 1) * 16, wc = (warp & 1) * 32;
    if (r0 + wr >= g.rhi || c0 + wc >= g.chi) return;
    const int tr = wr + (lane >> 3) * 4, tc = wc + (lane & 7) * 4;
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
        if (r >= g.rhi) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int c = c0 + tc + v;
            if (c < g.chi) F[(size_t)r * f + c] -= acc[u][v];
        }
    }
}

// FP32 trailing update with 128 x 128 tiles, 8 x 8 outputs per thread: the
// FP32 pipe is 64 times the FP64 one, so in single precision the update is
// bound by the tile's memory traffic and wants the larger tile (used for
// the large fronts; the 64 x 64 kernel above covers small ones and FP64).
constexpr int TB = 128;

__global__ void __launch_bounds__(THREADS) gemm128_kernel(DevPlan P, int node0, int k, int K0, int mode,
                                                         float *fronts) {
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    if (k >= n) return;
    const int nb = min(NB, n - k);
    const Region g = update_region(mode, k, nb, K0, n, f);
    const int r0 = g.rlo + blockIdx.y * TB, c0 = g.clo + blockIdx.x * TB;
    if (r0 >= g.rhi || c0 >= g.chi) return;
    float *F = fronts + P.front_off[node];
    __shared__ float As[NB][TB + 4];   // As[q][r]
    __shared__ float Bs[NB][TB + 4];   // Bs[q][c]
    for (int t = threadIdx.x; t < NB * TB; t += THREADS) {
        const int q = t % NB, r = t / NB;
        As[q][r] = (q < nb && r0 + r < g.rhi) ? F[(size_t)(r0 + r) * f + k + q] : 0.f;
    }
    for (int t = threadIdx.x; t < NB * TB; t += THREADS) {
        const int q = t / TB, c = t % TB;
        Bs[q][c] = (q < nb && c0 + c < g.chi) ? F[(size_t)(k + q) * f + c0 + c] : 0.f;
    }
    __syncthreads();
    const int tr = (threadIdx.x / 16) * 8, tc = (threadIdx.x % 16) * 8;
    float acc[8][8] = {};
#pragma unroll 4
    for (int q = 0; q < NB; ++q) {
        float a[8], b[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) { a[u] = As[q][tr + u]; b[u] = Bs[q][tc + u]; }
#pragma unroll
        for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[u][v] += a[u] * b[v];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int r = r0 + tr + u;
        if (r >= g.rhi) continue;
        float *row = F + (size_t)r * f;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int c = c0 + tc + v;
            if (c < g.chi) row[c] -= acc[u][v];
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
constexpr int TRI_WARPS = 4;
constexpr int TRI_THREADS = 32 * TRI_WARPS;
constexpr int GEMV_WARPS = 2;
constexpr int GEMV_THREADS = 32 * GEMV_WARPS;
constexpr int GEMV_ROWS = 32 * GEMV_WARPS;
constexpr int GEMV_TILES = 4;           // column tiles per warp
constexpr int GEMV_COLS = GEMV_TILES * SB;

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

DevPlan dev_plan(const tf_nd_plan *p, const int32_t *rank) {
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

int check_plan(const tf_nd_plan *p) {
    if (!p || p->n <= 0 || p->nnodes <= 0 || p->nlevels <= 0 || !p->level_ptr || !p->max_own || !p->max_f)
        return TF_ERR_ARG;
    if (!p->d_n_own || !p->d_f || !p->d_parent || !p->d_front_off || !p->d_idx_off || !p->d_idx ||
        !p->d_ea_off || !p->d_ea_map || !p->d_scat_pos || !p->d_scat_src || !p->d_piv_off || !p->d_rank)
        return TF_ERR_ARG;
    // the per-height launches put a height's fronts on a grid dimension
    // whose limit is 65535 (at 64^3 the widest height has 4097 fronts)
    for (int h = 0; h < p->nlevels; ++h)
        if (p->level_ptr[h + 1] - p->level_ptr[h] > 65535) return TF_ERR_SIZE;
    return TF_OK;
}

// Dynamic shared memory beyond a kernel's default limit (48 KiB minus its
// static shared memory) needs a per-kernel opt-in on the current device.
// Returns TF_ERR_SIZE when static plus dynamic shared memory would exceed
// what one CTA can have.
int ensure_smem(const void *kernel, size_t bytes) {
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

// One SIMT trailing update over a region of at most rows x cols per front.
template <typename T>
static void update(const DevPlan &D, int node0, int cnt, int k, int K0, int mode, int rows, int cols, T *fronts,
                   cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        if (rows >= 2 * TB || cols >= 2 * TB) {
            dim3 g((cols + TB - 1) / TB, (rows + TB - 1) / TB, cnt);
            gemm128_kernel<<<g, THREADS, 0, s>>>(D, node0, k, K0, mode, (float *)fronts);
            launched();
            return;
        }
    }
    dim3 g((cols + TN - 1) / TN, (rows + TM - 1) / TM, cnt);
    gemm_kernel<T><<<g, THREADS, 0, s>>>(D, node0, k, K0, mode, fronts);
    launched();
}

template <typename T>
int factor(const tf_nd_plan *p, const double *vals, T *fronts, int32_t *piv, int32_t *info, cudaStream_t s,
           const std::function<int(int)> *after_level) {
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
        // FP32 heights whose widest front has at least tc_min_front rows:
        // two-level blocking with the tensor-core update per outer block;
        // otherwise one level of rank-32 updates over the whole trailing front
        const bool two_level = sizeof(T) == 4 && p->tc_min_front > 0 && mf >= p->tc_min_front;
        const int bw = two_level ? KB : mo;
        const int mode = two_level ? UPD_COLS : UPD_ALL;
        const dim3 gl((mf + TRSM_THREADS - 1) / TRSM_THREADS, cnt, 2);
        for (int K0 = 0; K0 < mo; K0 += bw) {
            // the panels of the block; with two levels they update only the
            // block's own columns, so that the row swaps of later panels of
            // the block move rows whose other columns are all still untouched
            for (int k = K0; k < mo && k < K0 + bw; k += NB) {
                if ((e = panel<T>(D, node0, cnt, k, mo - k, nsm, fronts, piv, info, s))) return e;
                if (mf > 0) {
                    trsm_kernel<T><<<gl, TRSM_THREADS, 0, s>>>(D, node0, k, K0, mode, 0, fronts); launched();
                }
                const int rest = mf - k - 1;
                if (rest > 0) update<T>(D, node0, cnt, k, K0, mode, rest, two_level ? KB : rest, fronts, s);
            }
            if (!two_level) continue;
            // the block row right of the block, U[K0:E][E:f) = L_blk^-1 F[K0:E][E:f),
            // panel by panel after all of the block's swaps, then the rank-w
            // update of everything right of and below the block
            for (int k = K0; k < mo && k < K0 + KB; k += NB) {
                const dim3 gu((mf + TRSM_THREADS - 1) / TRSM_THREADS, cnt, 1);
                trsm_kernel<T><<<gu, TRSM_THREADS, 0, s>>>(D, node0, k, K0, UPD_ROWS, 1, fronts); launched();
                const int rest = mf - k - 1;
                if (rest > 0) update<T>(D, node0, cnt, k, K0, UPD_ROWS, KB, rest, fronts, s);
            }
            if constexpr (sizeof(T) == 4)
                if ((e = tc_update(D, node0, cnt, K0, mf, p->tc_terms == 1 ? 1 : 3, (float *)fronts, info, s)))
                    return e;
        }
        for (int rank = 0; rank < 2; ++rank) {
            dim3 ge(64, cnt);
            extend_add_kernel<T><<<ge, 256, 0, s>>>(D, node0, rank, fronts); launched();
        }
        if (after_level && (e = (*after_level)(h))) return e;
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
void bnd(const DevPlan &D, int node0, int cnt, int rows, int cols, const T *fronts, double *x, cudaStream_t s) {
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
        bnd<T, true>(D, node0, cnt, mf, mo, fronts, x, s);
    }
    for (int h = p->nlevels - 1; h >= 0; --h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        const int mo = p->max_own[h], mf = p->max_f[h];
        if (cnt <= 0 || mo <= 0) continue;
        bnd<T, false>(D, node0, cnt, mo, mf, fronts, x, s);
        if ((e = tri<T, false>(D, node0, cnt, mo, nsm, fronts, piv, x, s))) return e;
    }
    return cuda_status();
}

template int factor<float>(const tf_nd_plan *, const double *, float *, int32_t *, int32_t *, cudaStream_t,
                           const std::function<int(int)> *);
template int factor<double>(const tf_nd_plan *, const double *, double *, int32_t *, int32_t *, cudaStream_t,
                            const std::function<int(int)> *);
template void bnd<float, true>(const DevPlan &, int, int, int, int, const float *, double *, cudaStream_t);
template void bnd<float, false>(const DevPlan &, int, int, int, int, const float *, double *, cudaStream_t);
template void bnd<double, true>(const DevPlan &, int, int, int, int, const double *, double *, cudaStream_t);
template void bnd<double, false>(const DevPlan &, int, int, int, int, const double *, double *, cudaStream_t);

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" int tf_nd_factor_f64(const tf_nd_plan *plan, const double *d_vals, double *d_fronts, int32_t *d_piv,
                                int32_t *d_info, tf_stream_t stream) {
    return nd::factor<double>(plan, d_vals, d_fronts, d_piv, d_info, (cudaStream_t)stream, nullptr);
}

extern "C" int tf_nd_factor_f32(const tf_nd_plan *plan, const double *d_vals, float *d_fronts, int32_t *d_piv,
                                int32_t *d_info, tf_stream_t stream) {
    return nd::factor<float>(plan, d_vals, d_fronts, d_piv, d_info, (cudaStream_t)stream, nullptr);
}

extern "C" int tf_nd_solve_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv, double *d_x,
                               tf_stream_t stream) {
    return nd::solve<double>(plan, d_fronts, d_piv, d_x, (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv, double *d_x,
                               tf_stream_t stream) {
    return nd::solve<float>(plan, d_fronts, d_piv, d_x, (cudaStream_t)stream);
}
