// Application of the inverted factors (after tf_nd_invert_*) in one
// cooperative launch: the per-height products of tf_nd_solve_inv_* become
// phases of one kernel separated by grid-wide barriers instead of launches.
//
// Per tree height h, leaves first, then back from the root:
//   FA(h)  y = s + L11^-1 s           (s: own rows of x in pivot order)
//   FB(h)  x[bnd] -= L21 y
//   ...
//   BA(h)  t = y - U12 x[bnd];  x[own] = 0
//   BB(h)  x[own] += U11^-1 t
// Every phase is a set of independent 32 x 32 tiles of the fronts of one
// height.  Warps take tiles round-robin over the whole grid, double-buffer
// them with cp.async (the next tile and its 32 vector entries are fetched
// while the current one is multiplied), and every lane forms one row's
// partial dot product serially (no FP64 shuffles); partial sums of one row
// meet in global memory through atomics (y and t in the scratch vector, the
// boundary rows and, backward, the own rows in x).  Reads of values written
// in earlier phases bypass L1 (__ldcg).
//
// The launch is cooperative (all CTAs resident), so the barriers cannot
// deadlock; every barrier wait is still bounded: on giving up it raises the
// abort word (later waits return at once) and the sticky error word that
// tf_nd_sweep_status reports.
#include "tf_nd.cuh"

#include <algorithm>

namespace tf {
namespace nd {

constexpr int SW_WARPS = 8;
constexpr int SW_THREADS = 32 * SW_WARPS;
constexpr int SW_MAX_LEVELS = 64;
constexpr int SW_SPIN = 1 << 22;       // polls before a barrier wait gives up

enum : int { PH_FA = 0, PH_FB = 1, PH_BA = 2, PH_BB = 3 };

struct SweepLevel {
    int32_t node0, cnt, ns, nbs;      // fronts; own strips (max); boundary strips (max)
};

struct SweepArgs {
    int32_t nlevels;
    SweepLevel lv[SW_MAX_LEVELS];
};

// Workspace: int32 words [0] sticky error, [1] barrier count, [2] abort,
// then from byte 16 one double per front index entry (y, then t); all but
// the error word are cleared before every application.

__device__ __forceinline__ int sw_ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ void grid_barrier(int *words, int target) {
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(words + 1, 1);
        bool ok = false;
        for (int it = 0; it < SW_SPIN; ++it) {
            if (sw_ld_acquire(words + 1) >= target) { ok = true; break; }
            if (*(volatile int *)(words + 2)) break;
            __nanosleep(it < 64 ? 32 : 128);
        }
        if (!ok) {
            atomicExch(words + 2, 1);
            atomicExch(words, TF_ERR_TIMEOUT);
        }
        __threadfence();
    }
    __syncthreads();
}

// Lane l: sum_c buf[l][c] v[c] over c < l (lower) or c >= l (upper).
template <typename T>
__device__ __forceinline__ T sw_dot_tri(const T *buf, const T *v, int lane, bool lower) {
    T s = T(0);
#pragma unroll 8
    for (int c = 0; c < SB; ++c) {
        const bool keep = lower ? c < lane : c >= lane;
        s += (keep ? buf[lane * TSTRIDE + c] : T(0)) * v[c];
    }
    return s;
}

// Tiles of one phase: index -> (front slot q, row strip, column tile).
struct PhaseSpace {
    int ph, node0, cnt, ns, nbs, per, total;
};

__device__ __forceinline__ PhaseSpace phase_space(const SweepArgs &A, int ph, int h) {
    PhaseSpace P;
    const SweepLevel &L = A.lv[h];
    P.ph = ph; P.node0 = L.node0; P.cnt = L.cnt; P.ns = L.ns; P.nbs = L.nbs;
    if (ph == PH_FA || ph == PH_BB) P.per = L.ns * (L.ns + 1) / 2;
    else if (ph == PH_FB) P.per = L.nbs * L.ns;
    else P.per = L.ns * max(1, L.nbs);
    P.total = P.per * L.cnt;
    return P;
}

struct Tile {
    int node, n, f, r0, rmax, c0, cmax, diag;   // rows [r0, rmax), columns [c0, cmax) of the front
    bool zero;                                   // BA: the tile also clears x's own rows
};

// Decodes tile i; false when it lies outside its front.
__device__ __forceinline__ bool decode(const PhaseSpace &S, const DevPlan &P, int i, Tile &t) {
    const int q = i / S.per, rem = i % S.per;
    t.node = S.node0 + q;
    t.n = P.n_own[t.node];
    t.f = P.f[t.node];
    const int n = t.n, nb = t.f - t.n;
    int s, c;
    if (S.ph == PH_FA || S.ph == PH_BB) {
        // lower-triangle pair (a, b), b <= a, of the packed index
        int a = (int)((sqrtf(8.0f * rem + 1.0f) - 1.0f) * 0.5f);
        while ((a + 1) * (a + 2) / 2 <= rem) ++a;
        while (a * (a + 1) / 2 > rem) --a;
        const int b = rem - a * (a + 1) / 2;
        if (S.ph == PH_FA) { s = a; c = b; } else { s = b; c = a; }
        if (s * SB >= n || c * SB >= n) return false;
        t.r0 = s * SB; t.rmax = n; t.c0 = c * SB; t.cmax = n;
        t.diag = s == c;
        t.zero = false;
    } else if (S.ph == PH_FB) {
        s = rem / S.ns; c = rem % S.ns;
        if (s * SB >= nb || c * SB >= n) return false;
        t.r0 = n + s * SB; t.rmax = t.f; t.c0 = c * SB; t.cmax = n;
        t.diag = 0;
        t.zero = false;
    } else {
        const int nc = max(1, S.nbs);
        s = rem / nc; c = rem % nc;
        if (s * SB >= n || (c > 0 && c * SB >= nb)) return false;
        t.r0 = s * SB; t.rmax = n; t.c0 = n + c * SB; t.cmax = t.f;
        t.diag = 0;
        t.zero = c == 0;
    }
    return true;
}

template <typename T>
__global__ void __launch_bounds__(SW_THREADS, 1) sweep_kernel(DevPlan P, const T *fronts, const int32_t *piv,
                                                               double *x, double *ybuf, int *words,
                                                               const __grid_constant__ SweepArgs A) {
    extern __shared__ unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *buf0 = reinterpret_cast<T *>(smem_raw) + (2 * warp) * TILE;
    T *buf1 = buf0 + TILE;
    T *vsh = reinterpret_cast<T *>(smem_raw) + 2 * SW_WARPS * TILE + warp * 2 * SB;   // [2][32]
    const int gwarp = blockIdx.x * SW_WARPS + warp, nwarps = gridDim.x * SW_WARPS;
    const int nphase = 4 * A.nlevels;
    for (int p = 0; p < nphase; ++p) {
        const int ph = p < 2 * A.nlevels ? (p & 1) : 2 + (p & 1);
        const int h = p < 2 * A.nlevels ? p >> 1 : A.nlevels - 1 - ((p - 2 * A.nlevels) >> 1);
        const PhaseSpace S = phase_space(A, ph, h);
        Tile cur, nxt;
        int i = gwarp;
        while (i < S.total && !decode(S, P, i, cur)) i += nwarps;
        // the tile's vector entry for this lane (column c0 + lane)
        auto vload = [&](const Tile &t) -> T {
            const int c = t.c0 + lane;
            if (c >= t.cmax) return T(0);
            const int32_t *g = P.idx + P.idx_off[t.node];
            if (ph == PH_FA) return (T)__ldcg(x + g[piv[P.piv_off[t.node] + c]]);
            if (ph == PH_BA) return (T)__ldcg(x + g[c]);
            return (T)__ldcg(ybuf + P.idx_off[t.node] + c);
        };
        T vcur = T(0), vnxt = T(0);
        if (i < S.total) {
            tile_issue(buf0, fronts + P.front_off[cur.node], cur.f, cur.r0, cur.rmax, cur.c0, cur.cmax, lane);
            vcur = vload(cur);
        }
        for (int k = 0; i < S.total; ++k) {
            int j = i + nwarps;
            while (j < S.total && !decode(S, P, j, nxt)) j += nwarps;
            if (j < S.total) {
                tile_issue((k & 1) ? buf0 : buf1, fronts + P.front_off[nxt.node], nxt.f, nxt.r0, nxt.rmax, nxt.c0,
                           nxt.cmax, lane);
                vnxt = vload(nxt);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            T *v = vsh + (k & 1) * SB;
            v[lane] = vcur;
            __syncwarp();
            const T *b = (k & 1) ? buf1 : buf0;
            T acc = cur.diag ? sw_dot_tri(b, v, lane, ph == PH_FA) : tile_dot(b, v, lane);
            const int r = cur.r0 + lane;
            if (r < cur.rmax) {
                const int32_t *g = P.idx + P.idx_off[cur.node];
                double *yv = ybuf + P.idx_off[cur.node];
                if (ph == PH_FA) {
                    // the diagonal tile also adds s_r (column r is this tile's lane r)
                    double a = (double)acc;
                    if (cur.diag) a += (double)__ldcg(x + g[piv[P.piv_off[cur.node] + r]]);
                    atomicAdd(yv + r, a);
                } else if (ph == PH_FB) {
                    atomicAdd(x + g[r], -(double)acc);
                } else if (ph == PH_BA) {
                    atomicAdd(yv + r, -(double)acc);
                    if (cur.zero) x[g[r]] = 0.0;
                } else {
                    atomicAdd(x + g[r], (double)acc);
                }
            }
            __syncwarp();
            i = j;
            cur = nxt;
            vcur = vnxt;
        }
        if (p + 1 < nphase) grid_barrier(words, (p + 1) * gridDim.x);
    }
}

static size_t sweep_smem(int elem) {
    return (size_t)elem * (2 * SW_WARPS * TILE + SW_WARPS * 2 * SB);
}

// Heights h0 .. nlevels-1 go to the cooperative launch; the heights below
// (many fronts each, throughput-bound) keep their per-height launches
// before (forward) and after (backward) it.  top_heights <= 0 or >=
// nlevels: every height in the cooperative launch.
template <typename T>
static int solve_sweep(const tf_nd_plan *p, const T *fronts, const int32_t *piv, double *x, void *work,
                       size_t work_bytes, int top_heights, cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!fronts || !piv || !x || !work || work_bytes < 16) return TF_ERR_ARG;
    const int h0 = top_heights <= 0 || top_heights >= p->nlevels ? 0 : p->nlevels - top_heights;
    if (p->nlevels - h0 > SW_MAX_LEVELS) return TF_ERR_SIZE;
    SweepArgs A;
    A.nlevels = p->nlevels - h0;
    for (int i = 0; i < A.nlevels; ++i) {
        const int h = h0 + i;
        const int node0 = p->level_ptr[h], cnt = p->level_ptr[h + 1] - node0;
        const int mo = p->max_own[h], mf = p->max_f[h];
        A.lv[i].node0 = node0;
        A.lv[i].cnt = std::max(cnt, 0);
        A.lv[i].ns = (mo + SB - 1) / SB;
        // boundary rows of a front are at most f - n <= max_f of the height
        A.lv[i].nbs = (mf + SB - 1) / SB;
    }
    const size_t smem = sweep_smem(sizeof(T));
    if ((e = ensure_smem((const void *)sweep_kernel<T>, smem))) return e;
    int dev = 0, nsm = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sweep_kernel<T>, SW_THREADS, smem) != cudaSuccess)
        return TF_ERR_CUDA;
    if (occ < 1) return TF_ERR_SIZE;
    char *w = static_cast<char *>(work);
    int *words = reinterpret_cast<int *>(w);
    double *ybuf = reinterpret_cast<double *>(w + 16);
    // y / t accumulate through atomics: cleared with the barrier words (the
    // workspace holds one value per front index entry)
    if (cudaMemsetAsync(w + 4, 0, work_bytes - 4, s) != cudaSuccess) return TF_ERR_CUDA;
    launched();
    const DevPlan D = dev_plan(p, p->d_rank);
    if (h0 > 0 && (e = inv_levels<T>(p, D, fronts, piv, x, ybuf, h0, true, s))) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nsm * occ);
    cfg.blockDim = dim3(SW_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, sweep_kernel<T>, D, fronts, piv, x, ybuf, words, A) != cudaSuccess)
        return TF_ERR_CUDA;
    launched();
    if (h0 > 0 && (e = inv_levels<T>(p, D, fronts, piv, x, ybuf, h0, false, s))) return e;
    return cuda_status();
}

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" size_t tf_nd_sweep_workspace_bytes(const tf_nd_plan *plan) {
    if (nd::check_plan(plan)) return 0;
    int64_t idx_total = 0;
    if (cudaMemcpy(&idx_total, plan->d_idx_off + plan->nnodes, sizeof(int64_t), cudaMemcpyDeviceToHost) !=
        cudaSuccess)
        return 0;
    return 16 + 8 * (size_t)idx_total;
}

extern "C" int tf_nd_solve_sweep_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv,
                                     double *d_x, void *d_work, size_t work_bytes, int top_heights,
                                     tf_stream_t stream) {
    return nd::solve_sweep<double>(plan, d_fronts, d_piv, d_x, d_work, work_bytes, top_heights,
                                   (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_sweep_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv,
                                     double *d_x, void *d_work, size_t work_bytes, int top_heights,
                                     tf_stream_t stream) {
    return nd::solve_sweep<float>(plan, d_fronts, d_piv, d_x, d_work, work_bytes, top_heights,
                                  (cudaStream_t)stream);
}

extern "C" int tf_nd_sweep_status(void *d_work) {
    if (!d_work) return TF_ERR_ARG;
    int32_t err = 0;
    if (cudaMemcpy(&err, d_work, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess) return TF_ERR_CUDA;
    if (err != 0 && cudaMemset(d_work, 0, sizeof(err)) != cudaSuccess) return TF_ERR_CUDA;
    return err;
}
