// Explicit inverses of the factored own blocks (L11 unit lower, U11 upper)
// of every front, and the preconditioner application that uses them.
//
// Applying L11^-1 and U11^-1 by substitution is a chain of dependent 32-row
// block steps; on GB300, where a warp-wide FP64 instruction occupies an SM
// sub-partition for about 64 cycles, each step costs microseconds and the
// chains of the large fronts near the root dominate an application.  Both
// triangles are therefore inverted once per factorisation (in place: the
// inverse of the unit lower part keeps the strictly lower positions, the
// inverse of the upper part the upper ones), and an application becomes a
// triangular matrix-vector product (with the gather of its right-hand side
// folded in) and a boundary product per tree height and sweep, parallel over
// all rows.
//
// Inversion by recursive halving of each own block: a segment of m rows
// (m > 32) splits at m1 = 32 ceil(nb / 2) (nb = ceil(m / 32) row blocks),
//   L = [A 0; B C]:  L^-1 = [A^-1 0; -C^-1 B A^-1  C^-1]
//   U = [A B; 0 C]:  U^-1 = [A^-1  -A^-1 B C^-1; 0 C^-1]
// The 32-row diagonal blocks are inverted first (one warp each, column by
// column), then the off-diagonal blocks are combined from the deepest split
// up, two GEMMs per split (T = B X, B <- -Y T), batched over all splits of
// one depth and all fronts of one height.  The extra work is about n^3 / 3
// flops per triangle of an n-row own block.

#include "tf_nd.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

namespace tf {
namespace nd {

constexpr int IB = 32;        // diagonal block size
constexpr int IT = 32;        // GEMM tile (small: the top fronts' few splits must still fill the SMs)
constexpr int IK = 32;        // GEMM k chunk
constexpr int ITHREADS = 256;

__host__ __device__ constexpr int split_at(int m) { return IB * ((((m + IB - 1) / IB) + 1) / 2); }

// Scratch row stride for the products of a front with up to n own rows.
__host__ __device__ constexpr int inv_ld(int n) { return n > IB ? split_at(n) : 1; }

// Number of split depths of an n-row block (0 for a single 32-row block).
static int inv_depths(int n) {
    int d = 0;
    for (int nb = (n + IB - 1) / IB; nb > 1; nb = (nb + 1) / 2) ++d;
    return d;
}

// Segment of split node q at depth d; false when that node does not exist
// (a leaf was reached above it) or is a single block.
__device__ __forceinline__ bool split_node(int n, int depth, int q, int &r0, int &m) {
    r0 = 0;
    m = n;
    for (int d = depth - 1; d >= 0; --d) {
        if (m <= IB) return false;
        const int m1 = split_at(m);
        if ((q >> d) & 1) { r0 += m1; m -= m1; } else { m = m1; }
    }
    return m > IB;
}

// Invert the 32 x 32 diagonal blocks of every front of one height in place:
// the unit lower part (column j solves L x = e_j forwards, lane = column) and
// the upper part (U x = e_j backwards).  One warp per block.
template <typename T>
__global__ void __launch_bounds__(32) inv_diag_kernel(DevPlan P, int node0, T *fronts) {
    __shared__ T D[IB][IB + 1];
    __shared__ T X[IB][IB + 1];
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int b0 = blockIdx.x * IB;
    if (b0 >= n) return;
    const int nb = min(IB, n - b0);
    T *F = fronts + P.front_off[node] + (size_t)b0 * f + b0;
    const int lane = threadIdx.x;
    for (int i = 0; i < IB; ++i) D[i][lane] = (i < nb && lane < nb) ? F[(size_t)i * f + lane] : T(0);
    __syncwarp();
    // lower: x_i = [i == j] - sum_{t < i} L_it x_t
    for (int i = 0; i < IB; ++i) {
        T s = i == lane ? T(1) : T(0);
        for (int t = 0; t < i; ++t) s -= D[i][t] * X[t][lane];
        X[i][lane] = s;
    }
    __syncwarp();
    for (int i = 0; i < nb; ++i)
        if (lane < i) F[(size_t)i * f + lane] = X[i][lane];
    __syncwarp();
    // upper: x_i = ([i == j] - sum_{t > i} U_it x_t) / U_ii, one division per
    // row (lane i) instead of one per row and lane
    __shared__ T rdiag[IB];
    rdiag[lane] = lane < nb ? T(1) / D[lane][lane] : T(1);
    __syncwarp();
    for (int i = IB - 1; i >= 0; --i) {
        T s = i == lane ? T(1) : T(0);
        for (int t = i + 1; t < IB; ++t) s -= D[i][t] * X[t][lane];
        X[i][lane] = s * rdiag[i];
    }
    __syncwarp();
    for (int i = 0; i < nb; ++i)
        if (lane >= i && lane < nb) F[(size_t)i * f + lane] = X[i][lane];
}

// One GEMM of the recursive combination at split depth `depth` for every
// front of one height (grid: output tiles x split nodes x fronts):
//   UPPER = false, STAGE 0:  T = B A^-1        (m2 x m1, A^-1 unit lower)
//                  STAGE 1:  B = -C^-1 T       (C^-1 unit lower)
//   UPPER = true,  STAGE 0:  T = B C^-1        (m1 x m2, C^-1 upper)
//                  STAGE 1:  B = -A^-1 T       (A^-1 upper)
// with A = rows/cols [r0, r0+m1), C = [r0+m1, r0+m) of the node's segment,
// T in the front's scratch rows r0.. (row stride ld).  The triangular
// operand's zero half is skipped along k.
template <typename T, bool UPPER, int STAGE>
__global__ void __launch_bounds__(ITHREADS) inv_gemm_kernel(DevPlan P, int node0, int depth, T *fronts, T *work,
                                                            int ld, int64_t front_stride) {
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    int r0, m;
    if (!split_node(n, depth, blockIdx.y, r0, m)) return;
    const int m1 = split_at(m), m2 = m - m1;
    T *F = fronts + P.front_off[node];
    T *W = work + (int64_t)blockIdx.z * front_stride;
    // output M x N, inner K; operand accessors
    const int M = UPPER ? m1 : m2, N = UPPER ? m2 : m1, K = STAGE == 0 ? N : M;
    const int tiles_n = (N + IT - 1) / IT;
    const int tm = blockIdx.x / tiles_n, tn = blockIdx.x % tiles_n;
    const int i0 = tm * IT, j0 = tn * IT;
    if (i0 >= M) return;
    // k range with a nonzero triangular operand
    int klo = 0, khi = K;
    if (STAGE == 0) {        // (dense X) x (triangular Y): Y[k][j] nonzero for k >= j (lower) / k <= j (upper)
        if (UPPER) khi = min(K, j0 + IT); else klo = j0;
    } else {                 // (triangular Y) x (dense T): Y[i][k] nonzero for k <= i (lower) / k >= i (upper)
        if (UPPER) klo = i0; else khi = min(K, i0 + IT);
    }
    __shared__ T As[IK][IT + 1];   // As[k][i]
    __shared__ T Bs[IK][IT + 1];   // Bs[k][j]
    const int tr = (threadIdx.x / 16) * 2, tc = (threadIdx.x % 16) * 2;
    T acc[2][2] = {};
    for (int k0 = klo - (klo % IK); k0 < khi; k0 += IK) {
        for (int t = threadIdx.x; t < IK * IT; t += ITHREADS) {
            const int kk = t % IK, ii = t / IK;   // A tile: consecutive threads along k
            const int i = i0 + ii, k = k0 + kk;
            T a = T(0);
            if (i < M && k < K && k >= klo && k < khi) {
                if (STAGE == 0) {
                    a = UPPER ? F[(size_t)(r0 + i) * f + r0 + m1 + k] : F[(size_t)(r0 + m1 + i) * f + r0 + k];
                } else {
                    // triangular Y = (lower) C^-1 at [r0+m1, r0+m1) or (upper) A^-1 at [r0, r0)
                    const int base = UPPER ? r0 : r0 + m1;
                    if (UPPER) a = k > i ? F[(size_t)(base + i) * f + base + k] : (k == i ? F[(size_t)(base + i) * f + base + k] : T(0));
                    else a = k < i ? F[(size_t)(base + i) * f + base + k] : (k == i ? T(1) : T(0));
                }
            }
            As[kk][ii] = a;
        }
        for (int t = threadIdx.x; t < IK * IT; t += ITHREADS) {
            const int jj = t % IT, kk = t / IT;   // B tile: consecutive threads along j
            const int j = j0 + jj, k = k0 + kk;
            T b = T(0);
            if (j < N && k < K && k >= klo && k < khi) {
                if (STAGE == 0) {
                    // triangular Y = (lower) A^-1 at [r0, r0) or (upper) C^-1 at [r0+m1, r0+m1)
                    const int base = UPPER ? r0 + m1 : r0;
                    if (UPPER) b = k <= j ? F[(size_t)(base + k) * f + base + j] : T(0);
                    else b = k > j ? F[(size_t)(base + k) * f + base + j] : (k == j ? T(1) : T(0));
                } else {
                    b = W[(int64_t)(r0 + k) * ld + j];   // T (K x N) in scratch rows r0..
                }
            }
            Bs[kk][jj] = b;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < IK; ++kk) {
            T a[2], b[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) { a[u] = As[kk][tr + u]; b[u] = Bs[kk][tc + u]; }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int v = 0; v < 2; ++v) acc[u][v] += a[u] * b[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const int i = i0 + tr + u;
        if (i >= M) continue;
#pragma unroll
        for (int v = 0; v < 2; ++v) {
            const int j = j0 + tc + v;
            if (j >= N) continue;
            if (STAGE == 0)
                W[(int64_t)(r0 + i) * ld + j] = acc[u][v];
            else if (UPPER)
                F[(size_t)(r0 + i) * f + r0 + m1 + j] = -acc[u][v];
            else
                F[(size_t)(r0 + m1 + i) * f + r0 + j] = -acc[u][v];
        }
    }
}

// The same GEMMs for FP32 blocks with 128 x 128 output tiles (256 threads,
// 8 x 8 products per thread from two 16-byte shared-memory loads of each
// operand per k, k chunks of 16 double-buffered through registers): four
// times the products per shared-memory load of the 32 x 32 tiles, for the
// splits whose halves have at least 256 rows.
constexpr int JT = 128;
constexpr int JK = 16;
constexpr int JTHREADS = 256;

template <bool UPPER, int STAGE>
__global__ void __launch_bounds__(JTHREADS, 2) inv_gemm128_kernel(DevPlan P, int node0, int depth, float *fronts,
                                                                  float *work, int ld, int64_t front_stride) {
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    int r0, m;
    if (!split_node(n, depth, blockIdx.y, r0, m)) return;
    const int m1 = split_at(m), m2 = m - m1;
    float *F = fronts + P.front_off[node];
    float *W = work + (int64_t)blockIdx.z * front_stride;
    const int M = UPPER ? m1 : m2, N = UPPER ? m2 : m1, K = STAGE == 0 ? N : M;
    const int tiles_n = (N + JT - 1) / JT;
    const int tm = blockIdx.x / tiles_n, tn = blockIdx.x % tiles_n;
    const int i0 = tm * JT, j0 = tn * JT;
    if (i0 >= M) return;
    int klo = 0, khi = K;
    if (STAGE == 0) {
        if (UPPER) khi = min(K, j0 + JT); else klo = j0;
    } else {
        if (UPPER) klo = i0; else khi = min(K, i0 + JT);
    }
    if (klo >= khi) return;
    __shared__ __align__(16) float As[2][JK][JT + 4];   // As[k][i]
    __shared__ __align__(16) float Bs[2][JK][JT + 4];   // Bs[k][j]
    const int t = threadIdx.x;
    const int a_k = t % JK, a_i = t / JK;               // A loads: 16 k by 16 rows, 8 passes of 16 rows
    const int b_j = t % JT, b_k = t / JT;               // B loads: 128 j by 2 k, 8 passes of 2 k
    const int ty = t / 16, tx = t % 16;                 // products: rows ty*8.., columns tx*8..
    float ra[8], rb[8];
    auto gload = [&](int k0) {
        const int k = k0 + a_k;
        const bool kok = k >= klo && k < khi;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = i0 + a_i + 16 * q;
            float a = 0.f;
            if (kok && i < M) {
                if (STAGE == 0) {
                    a = UPPER ? F[(size_t)(r0 + i) * f + r0 + m1 + k] : F[(size_t)(r0 + m1 + i) * f + r0 + k];
                } else {
                    const int base = UPPER ? r0 : r0 + m1;
                    if (UPPER) a = k >= i ? F[(size_t)(base + i) * f + base + k] : 0.f;
                    else a = k < i ? F[(size_t)(base + i) * f + base + k] : (k == i ? 1.f : 0.f);
                }
            }
            ra[q] = a;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int kb = k0 + b_k + 2 * q, j = j0 + b_j;
            float b = 0.f;
            if (kb >= klo && kb < khi && j < N) {
                if (STAGE == 0) {
                    const int base = UPPER ? r0 + m1 : r0;
                    if (UPPER) b = kb <= j ? F[(size_t)(base + kb) * f + base + j] : 0.f;
                    else b = kb > j ? F[(size_t)(base + kb) * f + base + j] : (kb == j ? 1.f : 0.f);
                } else {
                    b = W[(int64_t)(r0 + kb) * ld + j];
                }
            }
            rb[q] = b;
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            As[buf][a_k][a_i + 16 * q] = ra[q];
            Bs[buf][b_k + 2 * q][b_j] = rb[q];
        }
    };
    float acc[8][8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
    const int kbeg = klo - (klo % JK);
    gload(kbeg);
    sstore(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = kbeg; k0 < khi; k0 += JK) {
        const bool more = k0 + JK < khi;
        if (more) gload(k0 + JK);
#pragma unroll
        for (int kk = 0; kk < JK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 8]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 8 + 4]);
            const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 8]);
            const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 8 + 4]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], b[v], acc[u][v]);
        }
        if (more) sstore(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int i = i0 + ty * 8 + u;
        if (i >= M) continue;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int j = j0 + tx * 8 + v;
            if (j >= N) continue;
            if (STAGE == 0)
                W[(int64_t)(r0 + i) * ld + j] = acc[u][v];
            else if (UPPER)
                F[(size_t)(r0 + i) * f + r0 + m1 + j] = -acc[u][v];
            else
                F[(size_t)(r0 + m1 + i) * f + r0 + j] = -acc[u][v];
        }
    }
}

static size_t invert_work_elems(const tf_nd_plan *p) {
    size_t w = 0;
    for (int h = 0; h < p->nlevels; ++h) {
        const int cnt = p->level_ptr[h + 1] - p->level_ptr[h], mo = p->max_own[h];
        if (cnt > 0 && mo > IB) w = std::max(w, (size_t)cnt * (size_t)mo * (size_t)inv_ld(mo));
    }
    return w;
}

// Inversion of the own blocks of the fronts of height h (scratch `work` of
// invert_work_elems elements, reused by every height).
template <typename T>
static void invert_level(const tf_nd_plan *p, const DevPlan &D, int h, T *fronts, T *work, cudaStream_t s) {
    const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
    const int mo = p->max_own[h];
    if (cnt <= 0 || mo <= 0) return;
    inv_diag_kernel<T><<<dim3((mo + IB - 1) / IB, cnt), 32, 0, s>>>(D, node0, fronts);
    launched();
    const int ld = inv_ld(mo);
    const int64_t stride = (int64_t)mo * ld;
    const int depths = inv_depths(mo);
    // largest segment at each split depth (the first half of a split is the
    // larger one), which bounds the tile grid of that depth
    std::vector<int> seg(depths + 1, mo);
    for (int d = 1; d <= depths; ++d) seg[d] = split_at(seg[d - 1]);
    for (int depth = depths - 1; depth >= 0; --depth) {
        const int half = split_at(seg[depth]);
        if constexpr (sizeof(T) == 4) {
            if (half >= 2 * JT) {
                const int tiles = ((half + JT - 1) / JT) * ((half + JT - 1) / JT);
                dim3 g(tiles, 1 << depth, cnt);
                inv_gemm128_kernel<false, 0><<<g, JTHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
                launched();
                inv_gemm128_kernel<false, 1><<<g, JTHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
                launched();
                inv_gemm128_kernel<true, 0><<<g, JTHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
                launched();
                inv_gemm128_kernel<true, 1><<<g, JTHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
                launched();
                continue;
            }
        }
        const int tiles = ((half + IT - 1) / IT) * ((half + IT - 1) / IT);
        dim3 g(tiles, 1 << depth, cnt);
        inv_gemm_kernel<T, false, 0><<<g, ITHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
        launched();
        inv_gemm_kernel<T, false, 1><<<g, ITHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
        launched();
        inv_gemm_kernel<T, true, 0><<<g, ITHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
        launched();
        inv_gemm_kernel<T, true, 1><<<g, ITHREADS, 0, s>>>(D, node0, depth, fronts, work, ld, stride);
        launched();
    }
}

template <typename T>
static int invert(const tf_nd_plan *p, const DevPlan &D, T *fronts, T *work, size_t work_bytes, cudaStream_t s) {
    if (work_bytes < invert_work_elems(p) * sizeof(T)) return TF_ERR_ARG;
    for (int h = 0; h < p->nlevels; ++h) invert_level<T>(p, D, h, fronts, work, s);
    return cuda_status();
}

// Factorisation on stream s with the inversion of each height's own blocks on
// stream aux as soon as that height is factored: the inversions (small,
// latency-bound launches) overlap the factorisation of the heights above,
// which near the root leaves most SMs idle.  The inversion of height h
// touches only the own blocks of height h, which nothing later in the
// factorisation reads.  aux joins s again before the return, also inside a
// stream capture.
template <typename T>
static int factor_invert(const tf_nd_plan *p, const double *vals, T *fronts, int32_t *piv, int32_t *info, T *work,
                         size_t work_bytes, cudaStream_t s, cudaStream_t aux) {
    if (work_bytes < invert_work_elems(p) * sizeof(T)) return TF_ERR_ARG;
    const DevPlan D = dev_plan(p, p->d_rank);
    std::vector<cudaEvent_t> ev(p->nlevels + 1, nullptr);
    int e = TF_OK;
    for (auto &x : ev)
        if (cudaEventCreateWithFlags(&x, cudaEventDisableTiming) != cudaSuccess) e = TF_ERR_CUDA;
    if (!e) {
        const std::function<int(int)> hook = [&](int h) -> int {
            if (cudaEventRecord(ev[h], s) != cudaSuccess || cudaStreamWaitEvent(aux, ev[h], 0) != cudaSuccess)
                return TF_ERR_CUDA;
            invert_level<T>(p, D, h, fronts, work, aux);
            return TF_OK;
        };
        e = factor<T>(p, vals, fronts, piv, info, s, &hook);
        if (cudaEventRecord(ev[p->nlevels], aux) != cudaSuccess ||
            cudaStreamWaitEvent(s, ev[p->nlevels], 0) != cudaSuccess)
            e = e ? e : TF_ERR_CUDA;
    }
    for (auto &x : ev)
        if (x) cudaEventDestroy(x);
    return e ? e : cuda_status();
}

// ---------------------------------------------------------------------------
// Application with inverted FP64 blocks (FP32 and BF16 factors: apply_kernel
// further down).  Per height, two launches per sweep:
//   forward   y = s + L11^-1 s into the scratch (s: the front's own rows of x
//             in pivot order, gathered by each CTA), then x[bnd] -= L21 y;
//   backward  t = y - U12 x[bnd] in the scratch, then x[own] = U11^-1 t.
// x's own rows are written only by the backward product, so no launch reads
// rows another CTA of the same launch writes.
// ---------------------------------------------------------------------------

constexpr int VT = 128;            // rows (one thread each) per CTA of the row kernel
constexpr int VW = 8;              // rows (one warp each) per CTA of the warp kernel

// One warp per row, lanes over the columns (coalesced reads of the row and
// of s), then a shuffle sum: five FP64 adds per row against the row's
// length / 32 products per lane, in exchange for spreading the large fronts
// near the root over many SMs.
template <typename S, bool FWD>
__global__ void __launch_bounds__(32 * VW) inv_apply_kernel(DevPlan P, int node0, const S *fronts,
                                                            const int32_t *piv, double *x, double *packed) {
    using T = S;
    extern __shared__ double s_gather[];   // forward: s[0 .. rmax), then their indices in x
    pdl_trigger();
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int rfirst = blockIdx.x * VW;
    if (rfirst >= n) return;
    const int32_t *g = P.idx + P.idx_off[node];
    double *pk = packed + P.idx_off[node];
    const double *sv = pk;
    {
        // the factors do not change during an application: start their
        // reads before waiting for the previous launch
        const int r = rfirst + (threadIdx.x >> 5), lane = threadIdx.x & 31;
        if (r < n) {
            const S *row = fronts + P.front_off[node] + (size_t)r * f;
            const int c0 = FWD ? 0 : r, c1 = FWD ? r : n;
            for (int c = c0 + lane * (128 / sizeof(S)); c < c1; c += 32 * (128 / sizeof(S))) prefetch_l2(row + c);
        }
    }
    // the positions in x of s (pivot order) do not depend on earlier launches
    const int rmax = min(n, rfirst + VW);
    int32_t *s_idx = reinterpret_cast<int32_t *>(s_gather + rmax);
    if (FWD) {
        const int32_t *pv = piv + P.piv_off[node];
        for (int c = threadIdx.x; c < rmax; c += 32 * VW) s_idx[c] = g[pv[c]];
    }
    pdl_wait();
    if (FWD) {
        for (int c = threadIdx.x; c < rmax; c += 32 * VW) s_gather[c] = x[s_idx[c]];
        __syncthreads();
        sv = s_gather;
    }
    const int lane = threadIdx.x & 31;
    const int r = rfirst + (threadIdx.x >> 5);
    if (r >= n) return;
    const S *row = fronts + P.front_off[node] + (size_t)r * f;
    const int c0 = FWD ? 0 : r, c1 = FWD ? r : n;
    T s0 = T(0), s1 = T(0);
    int c = c0 + lane;
#pragma unroll 4
    for (; c + 32 < c1; c += 64) {
        s0 += row[c] * (T)sv[c];
        s1 += row[c + 32] * (T)sv[c + 32];
    }
    if (c < c1) s0 += row[c] * (T)sv[c];
    T s = s0 + s1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (FWD) pk[r] = (double)s + sv[r];
        else x[g[r]] = (double)s;
    }
}

// The same product with one row per thread, for FP64 heights with many
// fronts whose own blocks are short (the leaves): there a warp's rows would
// be too short to pay for its FP64 shuffle sum, and the fronts alone fill the
// GPU.  Threads of a warp read the same s[c] (a broadcast) and their own rows
// through the L1 cache.
constexpr int VS = 128;            // own rows up to which a thread takes a row

template <typename T, bool FWD>
__global__ void __launch_bounds__(VT) inv_apply_rows_kernel(DevPlan P, int node0, const T *fronts,
                                                            const int32_t *piv, double *x, double *packed) {
    __shared__ double s_gather[VS];
    pdl_trigger();
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int32_t *g = P.idx + P.idx_off[node];
    double *pk = packed + P.idx_off[node];
    const double *sv = pk;
    if (threadIdx.x < n) {
        // this thread's row of the factors, before the wait
        const T *row = fronts + P.front_off[node] + (size_t)threadIdx.x * f;
        const int c0 = FWD ? 0 : threadIdx.x, c1 = FWD ? threadIdx.x : n;
        for (int c = c0; c < c1; c += 128 / sizeof(T)) prefetch_l2(row + c);
    }
    // the position in x of this thread's entry of s (pivot order) before the wait
    const int32_t xi = (FWD && threadIdx.x < n) ? g[piv[P.piv_off[node] + threadIdx.x]] : 0;
    pdl_wait();
    if (FWD) {
        if (threadIdx.x < n) s_gather[threadIdx.x] = x[xi];
        __syncthreads();
        sv = s_gather;
    }
    const int r = threadIdx.x;
    if (r >= n) return;
    const T *row = fronts + P.front_off[node] + (size_t)r * f;
    const int c0 = FWD ? 0 : r, c1 = FWD ? r : n;
    T s0 = T(0), s1 = T(0);
    int c = c0;
    #pragma unroll 4
    for (; c + 2 <= c1; c += 2) {
        s0 += row[c] * (T)sv[c];
        s1 += row[c + 1] * (T)sv[c + 1];
    }
    if (c < c1) s0 += row[c] * (T)sv[c];
    if (FWD) pk[r] = (double)(s0 + s1) + sv[r];
    else x[g[r]] = (double)(s0 + s1);
}

// Boundary couplings: forward x[bnd] -= L21 y (y from the scratch), backward
// t[own] -= U12 x[bnd] (into the scratch).  One 32-row by (32 ctiles)-column
// piece per warp (grid: row pieces x fronts x column pieces), tiles double
// buffered in shared memory, every lane one row; pieces of one row add
// through atomics.  Heights with few fronts take one tile per piece, so that
// their few large fronts still spread over many SMs.
constexpr int BV_WARPS = 2;
constexpr int BV_THREADS = 32 * BV_WARPS;
constexpr int BV_ROWS = 32 * BV_WARPS;
constexpr int BV_TILES = 4;        // most column tiles per piece

template <typename T, bool FWD>
__global__ void __launch_bounds__(BV_THREADS) inv_bnd_kernel(DevPlan P, int node0, int ctiles, const T *fronts,
                                                             double *x, double *packed) {
    extern __shared__ unsigned char smem_raw[];
    T *tiles = reinterpret_cast<T *>(smem_raw);   // [BV_WARPS][2] tiles
    __shared__ T v[BV_TILES * SB];
    pdl_trigger();
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int rlo = FWD ? n : 0, rhi = FWD ? f : n;
    const int clo = FWD ? 0 : n, chi = FWD ? n : f;
    const int ccols = ctiles * SB;
    const int rbase = rlo + blockIdx.x * BV_ROWS;
    const int cbase = clo + blockIdx.z * ccols;
    if (rbase >= rhi || cbase >= chi) return;
    const int cend = min(chi, cbase + ccols);
    const T *F = fronts + P.front_off[node];
    const int32_t *g = P.idx + P.idx_off[node];
    double *pk = packed + P.idx_off[node];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = rbase + warp * SB;
    T *b0 = tiles + (2 * warp) * TILE, *b1 = b0 + TILE;
    // the first two tiles of the factors and the vector's positions, before
    // waiting for the previous launch
    if (r0 < rhi) {
        tile_issue(b0, F, f, r0, rhi, cbase, chi, lane);
        if (cbase + SB < cend) tile_issue(b1, F, f, r0, rhi, cbase + SB, chi, lane);
    }
    constexpr int PER = BV_TILES * SB / BV_THREADS;
    int32_t vi[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int c = threadIdx.x + q * BV_THREADS;
        vi[q] = (c < ccols && cbase + c < cend) ? (FWD ? cbase + c : g[cbase + c]) : -1;
    }
    pdl_wait();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int c = threadIdx.x + q * BV_THREADS;
        if (c < ccols) v[c] = vi[q] >= 0 ? (T)(FWD ? pk[vi[q]] : x[vi[q]]) : T(0);
    }
    __syncthreads();
    if (r0 >= rhi) return;
    // tiles t and t + 1 are in flight while tile t is multiplied; tile t + 2
    // then goes into tile t's buffer
    T s = T(0);
    int t = 0;
    for (int c0 = cbase; c0 < cend; c0 += SB, ++t) {
        T *cur = (t & 1) ? b1 : b0;
        if (c0 + SB < cend)
            cp_async_wait<1>();
        else
            cp_async_wait<0>();
        __syncwarp();
        s += tile_dot_n(cur, v + (c0 - cbase), lane, cend - c0);
        __syncwarp();
        if (c0 + 2 * SB < cend) tile_issue(cur, F, f, r0, rhi, c0 + 2 * SB, chi, lane);
    }
    if (r0 + lane < rhi) {
        if (FWD) atomicAdd(x + g[r0 + lane], -(double)s);
        else atomicAdd(pk + r0 + lane, -(double)s);
    }
}

// ---------------------------------------------------------------------------
// Application with FP32 or BF16 factors (FP32 products, FP64 sums).  The own
// triangles and the boundary couplings are the same operation, a block of
// front rows times a vector over a range of columns, and one kernel does all
// four per height:
//   FTRI  y[r]      += s[r] + sum_{c<r}  L11^-1[r][c] s[c],  s[c] = x[g[piv[c]]]
//   FBND  x[g[r]]   -= sum_c L21[r][c] y[c]                  (r: boundary rows)
//   BBND  y[r]      -= sum_j U12[r][j] z[g[j]]               (j: boundary columns)
//   BTRI  z[g[r]]   += sum_{c>=r} U11^-1[r][c] y[c]
// y and z are vectors of the unknowns' length, addressed by the unknown
// (y[r] at g[r]), zeroed before the forward sweep; z is the result, copied
// into x after the backward sweep.  Every contribution is an atomic FP64 add,
// so a row may be split over any number of CTAs: the top fronts (16385 own
// rows at 64^3) spread over the whole GPU, and no CTA stages a vector in
// shared memory.  No launch reads an entry another CTA of the same launch
// writes.
//
// A warp owns AR rows and up to `ctiles` 32-column tiles of one front.  For
// each row its lanes load 32 consecutive columns (one coalesced segment;
// rows start at any alignment), multiply by the vector entry each lane holds
// for its column, and accumulate one partial sum per row; the next tile's
// loads are issued before the current tile's products, so a warp always has
// a tile in flight.  A butterfly of shuffles then leaves lane l with row
// (l mod AR)'s sum.  The factors are read with evict-first loads: they are
// streamed once per application, while the vectors and indices should stay
// in L2.  Five CTAs of four warps per SM (a register cap for six measured
// slightly slower: 5.38 against 5.29 ms per 64^3 application).
// ---------------------------------------------------------------------------
enum { AP_FTRI = 0, AP_FBND = 1, AP_BBND = 2, AP_BTRI = 3 };
constexpr int AR = 16;                  // rows per warp
constexpr int AWARPS = 4;
constexpr int ATHREADS = 32 * AWARPS;
constexpr int AROWS = AR * AWARPS;      // rows per CTA
constexpr int ACT = 16;                 // most column tiles per warp

__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const __nv_bfloat16 *p) { return __bfloat162float(__ldcs(p)); }

template <typename S, int KIND>
__global__ void __launch_bounds__(ATHREADS, 5) apply_kernel(DevPlan P, int node0, int ctiles, const S *fronts,
                                                         const int32_t *piv, const double *vin, double *vout) {
    constexpr bool LOWER = KIND == AP_FTRI, UPPER = KIND == AP_BTRI;
    pdl_trigger();
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const int rlo = KIND == AP_FBND ? n : 0, rhi = KIND == AP_FBND ? f : n;
    const int clo = KIND == AP_BBND ? n : 0, chi = KIND == AP_BBND ? f : n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r0 = rlo + blockIdx.x * AROWS + warp * AR;
    const int cbase = clo + blockIdx.z * ctiles * SB;
    if (r0 >= rhi || cbase >= chi) return;
    int cstart = cbase, cend = min(chi, cbase + ctiles * SB);
    // triangles: rows and columns both count from 0, so tiles are 32-aligned
    // relative to the rows; keep the tiles holding entries of the triangle
    if (LOWER) cend = min(cend, r0 + AR);                      // c <= r
    if (UPPER) cstart = max(cstart, r0 & ~(SB - 1));           // c >= r
    if (cstart >= cend) return;
    const int nrows = min(AR, rhi - r0);
    const int nt = (cend - cstart + SB - 1) / SB;
    const S *F = fronts + P.front_off[node] + (size_t)r0 * f;
    const int32_t *g = P.idx + P.idx_off[node];

    // entries of this warp's rows in tile c0 (zero outside the rows, the
    // column range and the triangle; L11's unit diagonal is added in FP64
    // at the end)
    auto load = [&](float (&d)[AR], int c0) {
        const int c = c0 + lane;
        const bool cok = c < cend;
        const bool diag = (LOWER || UPPER) && c0 + SB > r0 && c0 < r0 + AR;
        if (!diag) {
#pragma unroll
            for (int i = 0; i < AR; ++i) d[i] = (cok && i < nrows) ? ld_stream(F + (size_t)i * f + c) : 0.f;
        } else {
#pragma unroll
            for (int i = 0; i < AR; ++i) {
                const int r = r0 + i;
                const bool ok = cok && i < nrows && (LOWER ? c < r : c >= r);
                d[i] = ok ? ld_stream(F + (size_t)i * f + c) : 0.f;
            }
        }
    };

    // the vector entries of the warp's columns: positions before the wait,
    // values after it, in shared memory (one slot per lane and tile)
    __shared__ float vbuf[AWARPS][ACT * SB];
    float *vw = vbuf[warp];
    float cur[AR];
    load(cur, cstart);                         // the factors do not change: before the wait
    int32_t *vpos = reinterpret_cast<int32_t *>(vw);
    for (int t = 0; t < nt; ++t) {
        const int c = cstart + t * SB + lane;
        int32_t q = -1;
        if (c < cend) q = LOWER ? g[piv[P.piv_off[node] + c]] : g[c];
        vpos[t * SB + lane] = q;
    }
    const int32_t gout = lane < nrows ? g[r0 + lane] : 0;
    // FTRI: s[r] itself, when column r is in this warp's range
    const bool unit = LOWER && lane < nrows && r0 + lane >= cstart && r0 + lane < cend;
    const int32_t gdiag = unit ? g[piv[P.piv_off[node] + r0 + lane]] : 0;
    pdl_wait();
    for (int t = 0; t < nt; ++t) {
        const int32_t q = vpos[t * SB + lane];
        vw[t * SB + lane] = q >= 0 ? (float)vin[q] : 0.f;
    }
    float acc[AR];
#pragma unroll
    for (int i = 0; i < AR; ++i) acc[i] = 0.f;
#pragma unroll
    for (int t = 0; t < ACT; ++t) {
        if (t >= nt) break;
        float nxt[AR];
        if (t + 1 < nt) load(nxt, cstart + (t + 1) * SB);
        const float v = vw[t * SB + lane];
#pragma unroll
        for (int i = 0; i < AR; ++i) acc[i] = fmaf(cur[i], v, acc[i]);
        if (t + 1 < nt) {
#pragma unroll
            for (int i = 0; i < AR; ++i) cur[i] = nxt[i];
        }
    }
    // transpose-reduce: after the step with offset o a lane keeps o sums, the
    // half of its rows selected by its lane bit o; then the two half-warps
#pragma unroll
    for (int o = AR / 2; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int i = 0; i < o; ++i) {
            const float send = upper ? acc[i] : acc[i + o];
            const float keep = upper ? acc[i + o] : acc[i];
            acc[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
        }
    }
#pragma unroll
    for (int o = AR; o < 32; o <<= 1) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
    if (lane < nrows) {
        double sum = (double)acc[0];
        if (unit) sum += vin[gdiag];
        atomicAdd(vout + gout, (KIND == AP_FBND || KIND == AP_BBND) ? -sum : sum);
    }
}

// The factor entries an application reads -- every own row, and the own
// columns of the boundary rows -- converted from FP32 to BF16 (round to
// nearest) into a buffer with the fronts' layout.
__global__ void factors_to_bf16_kernel(DevPlan P, int node0, const float *fronts, __nv_bfloat16 *out) {
    const int node = node0 + blockIdx.y;
    const int n = P.n_own[node], f = P.f[node];
    const float *F = fronts + P.front_off[node];
    __nv_bfloat16 *O = out + P.front_off[node];
    const int64_t own = (int64_t)n * f, total = own + (int64_t)(f - n) * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t e;
        if (t < own) {
            e = t;
        } else {
            const int64_t u = t - own;
            e = (int64_t)(n + u / n) * f + u % n;
        }
        O[e] = __float2bfloat16_rn(F[e]);
    }
}

// The products of one application are launched with programmatic stream
// serialisation (pdl: every launch but the first of the sequence), so each
// starts reading its factors while the one before it finishes.  The three
// launchers below serve FP64 factors.
template <typename T, bool FWD>
static int inv_apply(const DevPlan &D, int node0, int cnt, int mo, const T *fronts, const int32_t *piv, double *x,
                     double *packed, bool pdl, cudaStream_t s) {
    cudaError_t ce = cudaSuccess;
    if (mo <= VS && cnt >= 256) {
        ce = launch_pdl(pdl, inv_apply_rows_kernel<T, FWD>, dim3(1, cnt), dim3(VT), 0, s, D, node0, fronts, piv, x,
                        packed);
    } else {
        const size_t sm = FWD ? (sizeof(double) + sizeof(int32_t)) * (size_t)mo : 0;
        if (sm > 48 * 1024) {
            const int e = ensure_smem((const void *)inv_apply_kernel<T, FWD>, sm);
            if (e) return e;
        }
        ce = launch_pdl(pdl, inv_apply_kernel<T, FWD>, dim3((mo + VW - 1) / VW, cnt), dim3(32 * VW), sm, s, D, node0,
                        fronts, piv, x, packed);
    }
    launched();
    return ce == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

template <typename T, bool FWD>
static int inv_bnd(const DevPlan &D, int node0, int cnt, int rows, int cols, int nsm, const T *fronts, double *x,
                   double *packed, bool pdl, cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return TF_OK;
    const int rb = (rows + BV_ROWS - 1) / BV_ROWS;
    const int wide = rb * cnt * ((cols + BV_TILES * SB - 1) / (BV_TILES * SB));
    const int ctiles = wide >= 4 * nsm ? BV_TILES : 1;
    dim3 grid(rb, cnt, (cols + ctiles * SB - 1) / (ctiles * SB));
    const cudaError_t ce = launch_pdl(pdl, inv_bnd_kernel<T, FWD>, grid, dim3(BV_THREADS),
                                      sizeof(T) * 2 * BV_WARPS * TILE, s, D, node0, ctiles, fronts, x, packed);
    launched();
    return ce == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// One product of the FP32 / BF16 application over every front of a height
// (at most `rows` rows and `cols` columns per front).  A warp takes up to ACT
// column tiles; fewer when the height would otherwise give the GPU fewer
// than `waves` warps per SM (the plan's apply_waves, 64 by default: about
// four waves of the 16-20 warps an SM holds).
template <typename S, int KIND>
static int apply_launch(const DevPlan &D, int node0, int cnt, int rows, int cols, int nsm, int waves,
                        const S *fronts, const int32_t *piv, const double *vin, double *vout, bool pdl,
                        cudaStream_t s) {
    if (rows <= 0 || cols <= 0) return TF_OK;
    constexpr bool TRI = KIND == AP_FTRI || KIND == AP_BTRI;
    const int64_t target = (int64_t)waves * nsm;
    int ct = ACT;
    for (; ct > 1; ct /= 2) {
        int64_t warps = (int64_t)((rows + AR - 1) / AR) * cnt * ((cols + ct * SB - 1) / (ct * SB));
        if (TRI) warps /= 2;
        if (warps >= target) break;
    }
    const dim3 grid((rows + AROWS - 1) / AROWS, cnt, (cols + ct * SB - 1) / (ct * SB));
    const cudaError_t ce = launch_pdl(pdl, apply_kernel<S, KIND>, grid, dim3(ATHREADS), 0, s, D, node0, ct, fronts,
                                      piv, vin, vout);
    launched();
    return ce == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

template <typename T>
int inv_levels(const tf_nd_plan *p, const DevPlan &D, const T *fronts, const int32_t *piv, double *x, double *packed,
               int h_end, bool fwd, cudaStream_t s) {
    int dev = 0, nsm = 0, e = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return TF_ERR_CUDA;
    h_end = std::min(h_end, p->nlevels);
    bool first = true;   // the sequence's first launch waits for everything before it
    for (int i = 0; i < h_end; ++i) {
        const int h = fwd ? i : h_end - 1 - i;
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        const int mo = p->max_own[h], mf = p->max_f[h];
        if (cnt <= 0 || mo <= 0) continue;
        if (fwd) {
            if ((e = inv_apply<T, true>(D, node0, cnt, mo, fronts, piv, x, packed, !first, s))) return e;
            if ((e = inv_bnd<T, true>(D, node0, cnt, mf, mo, nsm, fronts, x, packed, true, s))) return e;
        } else {
            if ((e = inv_bnd<T, false>(D, node0, cnt, mo, mf, nsm, fronts, x, packed, !first, s))) return e;
            if ((e = inv_apply<T, false>(D, node0, cnt, mo, fronts, piv, x, packed, true, s))) return e;
        }
        first = false;
    }
    return cuda_status();
}

// FP64 factors: the products above, with y / t in `packed`.
// FP32 and BF16 factors: apply_kernel, with y and z in the first 2n doubles
// of the scratch.
template <typename T>
static int solve_inv(const tf_nd_plan *p, const DevPlan &D, const T *fronts, const int32_t *piv, double *x,
                     double *scratch, cudaStream_t s) {
    if constexpr (sizeof(T) == 8) {
        int e = inv_levels<T>(p, D, fronts, piv, x, scratch, p->nlevels, true, s);
        return e ? e : inv_levels<T>(p, D, fronts, piv, x, scratch, p->nlevels, false, s);
    } else {
        int dev = 0, nsm = 0, e = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return TF_ERR_CUDA;
        const size_t n = (size_t)p->n;
        const int waves = p->apply_waves > 0 ? p->apply_waves : 64;
        double *y = scratch, *z = scratch + n;
        if (cudaMemsetAsync(scratch, 0, 2 * n * sizeof(double), s) != cudaSuccess) return TF_ERR_CUDA;
        bool first = true;   // the first launch waits for the memset
        for (int h = 0; h < p->nlevels; ++h) {
            const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
            const int mo = p->max_own[h], mf = p->max_f[h];
            if (cnt <= 0 || mo <= 0) continue;
            const int nb = cnt == 1 ? mf - mo : mf;     // boundary rows of a front, at most
            if ((e = apply_launch<T, AP_FTRI>(D, node0, cnt, mo, mo, nsm, waves, fronts, piv, x, y, !first, s)))
                return e;
            first = false;
            if ((e = apply_launch<T, AP_FBND>(D, node0, cnt, nb, mo, nsm, waves, fronts, piv, y, x, true, s)))
                return e;
        }
        for (int h = p->nlevels - 1; h >= 0; --h) {
            const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
            const int mo = p->max_own[h], mf = p->max_f[h];
            if (cnt <= 0 || mo <= 0) continue;
            const int nb = cnt == 1 ? mf - mo : mf;
            if ((e = apply_launch<T, AP_BBND>(D, node0, cnt, mo, nb, nsm, waves, fronts, piv, z, y, true, s)))
                return e;
            if ((e = apply_launch<T, AP_BTRI>(D, node0, cnt, mo, mo, nsm, waves, fronts, piv, y, z, true, s)))
                return e;
        }
        if (cudaMemcpyAsync(x, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return TF_ERR_CUDA;
        return cuda_status();
    }
}

template int inv_levels<double>(const tf_nd_plan *, const DevPlan &, const double *, const int32_t *, double *,
                                double *, int, bool, cudaStream_t);

// BF16 copy of the factor entries an application reads, one launch per height
static int factors_to_bf16(const tf_nd_plan *p, const float *fronts, __nv_bfloat16 *out, cudaStream_t s) {
    const DevPlan D = dev_plan(p, p->d_rank);
    for (int h = 0; h < p->nlevels; ++h) {
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        if (cnt <= 0) continue;
        const int64_t per = (int64_t)p->max_own[h] * p->max_f[h] * 2;
        const int bx = (int)std::min<int64_t>(std::max<int64_t>((per + 255) / 256, 1), 4096);
        factors_to_bf16_kernel<<<dim3(bx, cnt), 256, 0, s>>>(D, node0, fronts, out);
        launched();
    }
    return cuda_status();
}

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" size_t tf_nd_invert_workspace_bytes(const tf_nd_plan *plan, int elem_size) {
    if (!plan || (elem_size != 4 && elem_size != 8)) return 0;
    return nd::invert_work_elems(plan) * (size_t)elem_size;
}

extern "C" size_t tf_nd_solve_inv_workspace_bytes(const tf_nd_plan *plan) {
    if (nd::check_plan(plan)) return 0;
    int64_t len = 0;
    if (cudaMemcpy(&len, plan->d_idx_off + plan->nnodes, sizeof(len), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    // FP64 factors: one double per front index entry; FP32 / BF16: 2n
    return (size_t)std::max<int64_t>(len, 2 * (int64_t)plan->n) * sizeof(double);
}

extern "C" int tf_nd_factor_inv_f64(const tf_nd_plan *plan, const double *d_vals, double *d_fronts, int32_t *d_piv,
                                    int32_t *d_info, double *d_work, size_t work_bytes, tf_stream_t stream,
                                    tf_stream_t aux_stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_vals || !d_fronts || !d_piv || !aux_stream || aux_stream == stream ||
        (!d_work && nd::invert_work_elems(plan)))
        return TF_ERR_ARG;
    return nd::factor_invert<double>(plan, d_vals, d_fronts, d_piv, d_info, d_work, work_bytes, (cudaStream_t)stream,
                                     (cudaStream_t)aux_stream);
}

extern "C" int tf_nd_factor_inv_f32(const tf_nd_plan *plan, const double *d_vals, float *d_fronts, int32_t *d_piv,
                                    int32_t *d_info, float *d_work, size_t work_bytes, tf_stream_t stream,
                                    tf_stream_t aux_stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_vals || !d_fronts || !d_piv || !aux_stream || aux_stream == stream ||
        (!d_work && nd::invert_work_elems(plan)))
        return TF_ERR_ARG;
    return nd::factor_invert<float>(plan, d_vals, d_fronts, d_piv, d_info, d_work, work_bytes, (cudaStream_t)stream,
                                    (cudaStream_t)aux_stream);
}

extern "C" int tf_nd_invert_f64(const tf_nd_plan *plan, double *d_fronts, double *d_work, size_t work_bytes,
                                tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || (!d_work && nd::invert_work_elems(plan))) return TF_ERR_ARG;
    return nd::invert<double>(plan, nd::dev_plan(plan, plan->d_rank), d_fronts, d_work, work_bytes,
                              (cudaStream_t)stream);
}

extern "C" int tf_nd_invert_f32(const tf_nd_plan *plan, float *d_fronts, float *d_work, size_t work_bytes,
                                tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || (!d_work && nd::invert_work_elems(plan))) return TF_ERR_ARG;
    return nd::invert<float>(plan, nd::dev_plan(plan, plan->d_rank), d_fronts, d_work, work_bytes,
                             (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_inv_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv,
                                   double *d_x, double *d_scratch, tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || !d_piv || !d_x || !d_scratch) return TF_ERR_ARG;
    return nd::solve_inv<double>(plan, nd::dev_plan(plan, plan->d_rank), d_fronts, d_piv, d_x, d_scratch,
                                 (cudaStream_t)stream);
}

extern "C" int tf_nd_factors_to_bf16(const tf_nd_plan *plan, const float *d_fronts, uint16_t *d_out,
                                     tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || !d_out) return TF_ERR_ARG;
    return nd::factors_to_bf16(plan, d_fronts, reinterpret_cast<__nv_bfloat16 *>(d_out), (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_inv_bf16(const tf_nd_plan *plan, const uint16_t *d_fronts, const int32_t *d_piv,
                                    double *d_x, double *d_scratch, tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || !d_piv || !d_x || !d_scratch) return TF_ERR_ARG;
    return nd::solve_inv<__nv_bfloat16>(plan, nd::dev_plan(plan, plan->d_rank),
                                        reinterpret_cast<const __nv_bfloat16 *>(d_fronts), d_piv, d_x, d_scratch,
                                        (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_inv_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv,
                                   double *d_x, double *d_scratch, tf_stream_t stream) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_fronts || !d_piv || !d_x || !d_scratch) return TF_ERR_ARG;
    return nd::solve_inv<float>(plan, nd::dev_plan(plan, plan->d_rank), d_fronts, d_piv, d_x, d_scratch,
                                (cudaStream_t)stream);
}
