// Panel factorisations of the nested-dissection multifrontal LU (the rest of
// the factorisation and the solves are in tf_nd.cu).  Included by
// tf_nd_panel_f32.cu and tf_nd_panel_f64.cu, which instantiate one precision
// each so that the two compile in parallel.
#pragma once

#include "tf_nd.cuh"

#include <mutex>

namespace tf {
namespace nd {

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

// Distributed-shared-memory messages: st.async stores into another CTA of
// the cluster and signals the bytes on that CTA's mbarrier, whose phase
// completes once the expected bytes (and its one local arrival) are in.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned cluster_addr(unsigned a, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_async(unsigned raddr, double v, unsigned rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];\n"
                 ::"r"(raddr), "l"(__double_as_longlong(v)), "r"(rbar) : "memory");
}
__device__ __forceinline__ void st_async(unsigned raddr, float v, unsigned rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];\n"
                 ::"r"(raddr), "r"(__float_as_uint(v)), "r"(rbar) : "memory");
}
__device__ __forceinline__ void st_async(unsigned raddr, int v, unsigned rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];\n"
                 ::"r"(raddr), "r"(v), "r"(rbar) : "memory");
}
__device__ __forceinline__ void mbar_init(void *bar, unsigned count) {
    asm volatile("mbarrier.init.shared.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(void *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait for the given phase parity; false if it gave up.
__device__ __forceinline__ bool mbar_wait(void *bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    for (int it = 0; it < (1 << 22); ++it) {
        unsigned ok;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}

// Pivot-search key of an entry: the IEEE-754 bit pattern of |v| (non-negative
// floating-point values order like their bit patterns), with NaN mapped to 0,
// so that the searches compare on the integer pipe and leave the scarce FP64
// pipe to the eliminations.  Rows that may not be chosen get key -1.
__device__ __forceinline__ long long mag_key(double v) {
    const long long b = __double_as_longlong(v) & 0x7fffffffffffffffll;
    return b > 0x7ff0000000000000ll ? 0 : b;
}
__device__ __forceinline__ long long mag_key(float v) {
    const int b = __float_as_int(v) & 0x7fffffff;
    return b > 0x7f800000 ? 0 : b;
}
__device__ __forceinline__ void st_async(unsigned raddr, long long v, unsigned rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];\n"
                 ::"r"(raddr), "l"(v), "r"(rbar) : "memory");
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
    __shared__ int cur[2 * NB];    // composition scratch (shared: indexed at run time)
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
    __shared__ long long wval[NW];
    __shared__ int widx[NW];
    __shared__ T lstage[NB];
    __shared__ long long cval[2][CL];   // candidates' pivot-search keys
    __shared__ T crcp[2][CL];      // 1 / (candidate's entry in column lc)
    __shared__ int cidx[2][CL];
    __shared__ T crow[2][CL][NB];
    __shared__ T lrow[2][NB];
    __shared__ int s_piv[NB];
    __shared__ __align__(8) unsigned long long mbar[2];
    // bytes each CTA receives per column: every CTA's candidate (row, value,
    // index, reciprocal pivot) and the diagonal row
    constexpr unsigned TX = CL * (NB * sizeof(T) + sizeof(T) + sizeof(long long) + sizeof(int)) + NB * sizeof(T);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int my = lo + threadIdx.x;
    const bool have = my < hi;
    if (threadIdx.x == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    cluster.sync();   // every CTA's barriers exist before the first message
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
            long long best = (have && my >= lc) ? mag_key(a[lc]) : -1ll;
            int bi = (have && my >= lc) ? my : 0x7fffffff;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
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
            if (threadIdx.x == 0) mbar_expect_tx(&mbar[par], TX);
            __syncthreads();
            if (warp == 0) {
                long long b = wval[0];
                int i = widx[0], ws = 0;
                for (int w = 1; w < NW; ++w)
                    if (wval[w] > b || (wval[w] == b && widx[w] < i)) { b = wval[w]; i = widx[w]; ws = w; }
                const T v = i < rows ? wrow[ws][lane] : T(0);
                T rcp = T(0);
                if (lane == lc) rcp = T(1) / (v == T(0) ? T(1e-30) : v);   // singular pivot: flagged through info
                for (int d = 0; d < CL; ++d) {
                    const unsigned rb = cluster_addr(smem_u32(&mbar[par]), d);
                    st_async(cluster_addr(smem_u32(&crow[par][q][lane]), d), v, rb);
                    if (lane == 0) {
                        st_async(cluster_addr(smem_u32(&cval[par][q]), d), b, rb);
                        st_async(cluster_addr(smem_u32(&cidx[par][q]), d), i, rb);
                    }
                    if (lane == lc) st_async(cluster_addr(smem_u32(&crcp[par][q]), d), rcp, rb);
                }
            } else if (warp == 1 && q == ql) {
                const T v = lstage[lane];
                for (int d = 0; d < CL; ++d)
                    st_async(cluster_addr(smem_u32(&lrow[par][lane]), d), v, cluster_addr(smem_u32(&mbar[par]), d));
            }
            if (!mbar_wait(&mbar[par], (lc >> 1) & 1) && threadIdx.x == 0 && info)
                atomicAdd(info, 1 << 20);   // gave up waiting: reported as a failed factorisation
            long long b = -1;
            int r = 0x7fffffff, w = 0;
#pragma unroll
            for (int c = 0; c < CL; ++c)
                if (cval[par][c] > b || (cval[par][c] == b && cidx[par][c] < r)) { b = cval[par][c]; r = cidx[par][c]; w = c; }
            const T *prow = crow[par][w];
            T rp = crcp[par][w];
            if (r >= rows) {   // no candidate row (cannot happen while lc < rows)
                r = lc;
                b = 0;
                prow = lrow[par];
                rp = T(1) / prow[lc];
            }
            if (threadIdx.x == 0) {
                s_piv[lc] = r;
                if (q == 0) {
                    pv[k + lc] = k + r;
                    if (b == 0 && info) atomicAdd(info, 1);   // zero (or NaN) pivot
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

// Panel launch over a cluster of CL CTAs per front.  Returns TF_ERR_SIZE when
// the per-CTA share of the panel does not fit in shared memory.
template <typename T, int CL>
static int launch_panel(const DevPlan &D, int node0, int cnt, int k, int rows, T *fronts, int32_t *piv,
                        int32_t *info, cudaStream_t s) {
    const size_t sm = sizeof(T) * (size_t)((rows + CL - 1) / CL) * PSTRIDE;
    const int e = ensure_smem((const void *)panel_cluster_kernel<T, CL>, sm);
    if (e) return e;
    if (CL > 8) {
        // clusters of more than 8 CTAs are a per-kernel opt-in
        static std::mutex mu;
        std::lock_guard<std::mutex> lock(mu);
        if (cudaFuncSetAttribute((const void *)panel_cluster_kernel<T, CL>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            return TF_ERR_SIZE;
        }
        // a cluster this large needs that many free SMs in one GPC
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL);
        cfg.blockDim = dim3(THREADS);
        cfg.dynamicSmemBytes = sm;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, (const void *)panel_cluster_kernel<T, CL>, &cfg) !=
                cudaSuccess ||
            clusters < 1) {
            cudaGetLastError();
            return TF_ERR_SIZE;
        }
    }
    panel_cluster_kernel<T, CL><<<cnt * CL, THREADS, sm, s>>>(D, node0, k, fronts, piv, info);
    launched();
    return TF_OK;
}

// Cluster size for cnt fronts with up to `rows` panel rows: about one CTA per
// SM in total and at least 32 rows per CTA.
static int panel_cluster_size(int cnt, int rows, int nsm, int clmax) {
    int cl = clmax;
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

// One thread block size (256 rows per CTA) keeps the number of fully
// unrolled instantiations, and so the build time, small.
constexpr int PANEL_PT = 256;

template <typename T, int CL>
static int launch_panel_reg_pt(const DevPlan &D, int node0, int cnt, int k, int rows, T *fronts, int32_t *piv,
                               int32_t *info, cudaStream_t s) {
    // the many small fronts near the leaves: 128-thread CTAs, twice as many
    // resident per SM to hide the per-column latency
    if constexpr (CL == 1)
        if (rows <= PANEL_PT / 2) return launch_panel_reg<T, 1, PANEL_PT / 2>(D, node0, cnt, k, fronts, piv, info, s);
    if ((rows + CL - 1) / CL <= PANEL_PT) return launch_panel_reg<T, CL, PANEL_PT>(D, node0, cnt, k, fronts, piv, info, s);
    return TF_ERR_SIZE;
}

template <typename T>
int panel(const DevPlan &D, int node0, int cnt, int k, int rows, int nsm, T *fronts, int32_t *piv,
                 int32_t *info, cudaStream_t s) {
    // one register-held row per thread while a cluster of up to 8 CTAs
    // offers at most 512 rows per CTA
    // register panels: up to 4 CTAs, measured faster than 8 at 256^2 (fewer
    // messages per column; the extra rows per CTA cost less than the exchange)
    for (int cl = panel_cluster_size(cnt, rows, nsm, 4); cl <= 8; cl *= 2) {
        int e = TF_ERR_SIZE;
        switch (cl) {
        case 1: e = launch_panel_reg_pt<T, 1>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 2: e = launch_panel_reg_pt<T, 2>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 4: e = launch_panel_reg_pt<T, 4>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        default: e = launch_panel_reg_pt<T, 8>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        }
        if (e != TF_ERR_SIZE) return e;
    }
    // larger panels: rows staged in shared memory, spread over up to 8 CTAs,
    // or 16 (a non-portable cluster size) for the tallest FP32 panels
    for (int cl = panel_cluster_size(cnt, rows, nsm, 8); cl <= 16; cl *= 2) {
        int e = TF_ERR_SIZE;
        switch (cl) {
        case 1: e = launch_panel<T, 1>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 2: e = launch_panel<T, 2>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 4: e = launch_panel<T, 4>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        case 8: e = launch_panel<T, 8>(D, node0, cnt, k, rows, fronts, piv, info, s); break;
        default:
            if constexpr (sizeof(T) == 4)
                if (cnt * 16 <= nsm) e = launch_panel<T, 16>(D, node0, cnt, k, rows, fronts, piv, info, s);
            break;
        }
        if (e != TF_ERR_SIZE) return e;
    }
    panel_kernel<T><<<cnt, THREADS, 0, s>>>(D, node0, k, fronts, piv, info);
    launched();
    return TF_OK;
}


}  // namespace nd
}  // namespace tf
