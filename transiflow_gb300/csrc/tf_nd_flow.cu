// Dataflow application of the inverted factors (after tf_nd_invert_*): the
// forward and the backward sweep of every front in ONE persistent launch.
//
// The height-by-height application (tf_nd_solve_inv_*) issues a product with
// the inverted own block and a boundary product per height and sweep.  Near
// the root each of those launches holds a handful of fronts and most SMs wait
// for the launch boundary.  Here the work is a list of tasks in
// an order compatible with the elimination tree; CTAs take tasks in list order
// from an atomic ticket, and a task waits (bounded spin) only for the tasks it
// depends on, through per-front counters:
//
//   forward  own rows   y = s + L11^-1 s  (s: own rows of x, permuted),
//            waits for the boundary products of the front's children;
//            boundary   x[bnd] -= L21 y, waits for the front's own-row tasks;
//   backward boundary   t = y - U12 x[bnd], waits for the parent front's
//                       backward own-row tasks (the root: its forward);
//            own rows   x[own] = U11^-1 t, waits for the front's boundary tasks.
//
// Fronts whose factors fit in few tiles go to bundle tasks: up to FW fronts
// of one height, one warp each doing both parts of the sweep.  The other
// tasks cover up to FSPT 32-row strips of one front; the CTA's 8 warps share
// the (strip, tile) pairs.  Each warp double-buffers 32 x 32 tiles with
// cp.async and every lane forms one row's dot product serially (no FP64
// shuffles).  Tiles are issued before the dependency wait: the factors do not
// change during the launch.  (Opt-in: the per-height launches measured faster.)
//
// Deadlock freedom does not depend on how many CTAs are resident: a task only
// waits for tasks earlier in the list, which were taken by CTAs already
// running.  Every wait gives up after a bounded number of polls; it then sets
// the abort word (all later waits return at once) and the sticky error word
// that tf_nd_flow_status reports.
#include "tf_nd.cuh"

#include <algorithm>
#include <vector>

namespace tf {
namespace nd {

constexpr int FW = 8;                  // warps per CTA
constexpr int FTHREADS = 32 * FW;
constexpr int FSPT = 4;                // most 32-row strips per task
constexpr int FLOW_SPIN = 1 << 22;     // polls before a wait gives up

// Task kinds.  Split fronts: one CTA per task, a range of 32-row strips of
// one part of a sweep.  Small fronts: bundles of up to FW fronts of one
// height, one warp per front doing its whole sweep (r0 = number of fronts).
enum : int { K_FOWN = 0, K_FBND = 1, K_BBND = 3, K_BOWN = 4, K_WFWD = 5, K_WBWD = 6 };
constexpr int FUSE_F = 512;            // widest front a warp task takes

struct FlowTask {
    int32_t node, kind, r0, r1;        // front rows [r0, r1) (split tasks)
    int32_t wait, target, signal, pad; // counter waited for (>= target) / incremented, -1: none
};

// Per-front counters of the bundles (the warp tasks read them per front).
struct NodeFlow {
    int32_t fw_wait, fw_target, fw_signal, bw_wait, bw_target, bw_signal, pad0, pad1;
};

// Device workspace: header, four counters per front, y/t values (one per
// front index entry), per-front bundle counters, tasks.  Bytes
// [FLOW_RESET_OFF, counters end) are cleared before every application.
struct FlowHeader {
    int32_t err, ntasks, pad0, pad1;
    int64_t tasks_off, ybuf_off, nodes_off;
    int32_t abort, ticket, pad2, pad3;
};
static_assert(sizeof(FlowHeader) == 56, "flow header layout");
constexpr size_t FLOW_RESET_OFF = 40;
enum { C_FA = 0, C_KIDS = 1, C_BA = 2, C_BWD = 3 };   // counters of front i: 4 i + C_*

__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Polls *ctr until it reaches target; false when the wait gave up (or
// another wait did).
__device__ bool flow_wait(const int *ctr, int target, int *abort) {
    for (int it = 0; it < FLOW_SPIN; ++it) {
        if (ld_acquire(ctr) >= target) return true;
        if (*(volatile int *)abort) return false;
        __nanosleep(it < 32 ? 32 : 256);
    }
    return false;
}

// Rows [rlo, rhi) of one 32-row strip, its column range [c0, cmax) in 32-wide
// tiles, and the tile holding the diagonal (-1: none).
struct Strip {
    int rhi, c0, cmax, ntiles, diag;
};

__device__ __forceinline__ Strip strip_of(int kind, int n, int f, int R) {
    Strip s;
    if (kind == K_FOWN) {            // L11^-1 (strictly lower part)
        s.rhi = min(R + SB, n); s.c0 = 0; s.cmax = n; s.ntiles = R / SB + 1; s.diag = R / SB;
    } else if (kind == K_FBND) {     // L21
        s.rhi = min(R + SB, f); s.c0 = 0; s.cmax = n; s.ntiles = (n + SB - 1) / SB; s.diag = -1;
    } else if (kind == K_BBND) {     // U12
        s.rhi = min(R + SB, n); s.c0 = n; s.cmax = f; s.ntiles = (f - n + SB - 1) / SB; s.diag = -1;
    } else {                         // U11^-1 (upper part with the diagonal)
        s.rhi = min(R + SB, n); s.c0 = R; s.cmax = n; s.ntiles = (n - R + SB - 1) / SB; s.diag = 0;
    }
    return s;
}

// Lane l: sum_c buf[l][c] v[c] over c < l (lower) or c >= l (upper).
template <typename T>
__device__ __forceinline__ T tile_dot_tri(const T *buf, const T *v, int lane, bool lower) {
    T s = T(0);
#pragma unroll 8
    for (int c = 0; c < SB; ++c) {
        const bool keep = lower ? c < lane : c >= lane;
        s += (keep ? buf[lane * TSTRIDE + c] : T(0)) * v[c];
    }
    return s;
}

// The (strip, tile) pairs of `ns` strips starting at row R0, strip-major; a
// cursor that moves forward only.
struct Cursor {
    int kind, n, f, R0, ns, s, base;
    __device__ bool locate(int it, int &si, int &ti) {
        while (s < ns) {
            const int nt = strip_of(kind, n, f, R0 + s * SB).ntiles;
            if (it < base + nt) {
                si = s;
                ti = it - base;
                return true;
            }
            base += nt;
            ++s;
        }
        return false;
    }
};

template <typename T>
__device__ __forceinline__ void issue_item(int kind, int n, int f, int R0, int si, int ti, const T *F, T *buf,
                                           int lane) {
    const int R = R0 + si * SB;
    const Strip g = strip_of(kind, n, f, R);
    tile_issue(buf, F, f, R, g.rhi, g.c0 + ti * SB, g.cmax, lane);
}

// Starts the copy of this warp's first tile of the strips at R0.
template <typename T>
__device__ void products_prefetch(int kind, int n, int f, int R0, int ns, const T *F, T *tiles) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Cursor cur{kind, n, f, R0, ns, 0, 0};
    int si, ti;
    if (cur.locate(warp, si, ti)) issue_item(kind, n, f, R0, si, ti, F, tiles + (2 * warp) * TILE, lane);
}

// Per-warp partial row sums of `ns` strips into red[warp][strip][lane]; the
// vector holds column c at vec[c - vbase] (zero past its end, up to the
// next multiple of 32).  `issued`: the first tile is already in flight.
template <typename T>
__device__ __forceinline__ void products(int kind, int n, int f, int R0, int ns, const T *F, const T *vec, int vbase, T *tiles,
                         T *red, bool issued) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T *buf0 = tiles + (2 * warp) * TILE, *buf1 = buf0 + TILE;
    for (int s = 0; s < ns; ++s) red[(warp * FSPT + s) * SB + lane] = T(0);
    Cursor cur{kind, n, f, R0, ns, 0, 0};
    int it = warp, si, ti;
    if (!cur.locate(it, si, ti)) return;
    if (!issued) issue_item(kind, n, f, R0, si, ti, F, buf0, lane);
    T acc = T(0);
    int accs = si;
    for (int k = 0;; ++k) {
        int sn = 0, tn = 0;
        const bool more = cur.locate(it + FW, sn, tn);
        if (more) {
            issue_item(kind, n, f, R0, sn, tn, F, (k & 1) ? buf0 : buf1, lane);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const T *b = (k & 1) ? buf1 : buf0;
        const Strip g = strip_of(kind, n, f, R0 + si * SB);
        const T *v = vec + (g.c0 + ti * SB - vbase);
        const T d = ti == g.diag ? tile_dot_tri(b, v, lane, kind == K_FOWN) : tile_dot(b, v, lane);
        __syncwarp();
        if (si != accs) {
            red[(warp * FSPT + accs) * SB + lane] = acc;
            acc = T(0);
            accs = si;
        }
        acc += d;
        if (!more) break;
        it += FW;
        si = sn;
        ti = tn;
    }
    red[(warp * FSPT + accs) * SB + lane] = acc;
}

// Everything one task needs to know about its front.
template <typename T>
struct Front {
    int node, n, f;
    const T *F;
    const int32_t *g, *pv;
    double *y;
};

template <typename T>
__device__ __forceinline__ Front<T> front_of(const DevPlan &P, int node, const T *fronts, const int32_t *piv,
                                             double *ybuf) {
    Front<T> fr;
    fr.node = node;
    fr.n = P.n_own[node];
    fr.f = P.f[node];
    fr.F = fronts + P.front_off[node];
    fr.g = P.idx + P.idx_off[node];
    fr.pv = piv + P.piv_off[node];
    fr.y = ybuf + P.idx_off[node];
    return fr;
}

// The kind's update of x / y for row r, given the row's product sum; `out`
// (tasks doing both parts of a sweep) receives y or t for the next part.
template <typename T>
__device__ __forceinline__ void row_out(int kind, const Front<T> &fr, int r, T sum, T *out, double *x) {
    if (kind == K_FOWN) {
        const double yr = (double)sum + __ldcg(x + fr.g[fr.pv[r]]);
        fr.y[r] = yr;
        if (out) out[r] = (T)yr;
    } else if (kind == K_FBND) {
        atomicAdd(x + fr.g[r], -(double)sum);
    } else if (kind == K_BBND) {
        const double tr = __ldcg(fr.y + r) - (double)sum;
        if (out) out[r] = (T)tr;
        else fr.y[r] = tr;
    } else {
        x[fr.g[r]] = (double)sum;
    }
}

// CTA task: rows [Rb, Re) of one kind in chunks of FSPT strips; products
// shared by the warps, then the sum over warps.
template <typename T>
__device__ __forceinline__ void run_rows(int kind, const Front<T> &fr, int Rb, int Re, const T *vec, int vbase, T *tiles, T *red,
                         double *x, bool issued) {
    for (int R0 = Rb; R0 < Re; R0 += FSPT * SB) {
        const int ns = min(FSPT, (Re - R0 + SB - 1) / SB);
        products(kind, fr.n, fr.f, R0, ns, fr.F, vec, vbase, tiles, red, issued && R0 == Rb);
        __syncthreads();
        const int t = threadIdx.x;
        if (t < ns * SB) {
            const int s = t >> 5, l = t & 31;
            T sum = T(0);
#pragma unroll
            for (int w = 0; w < FW; ++w) sum += red[(w * FSPT + s) * SB + l];
            const int r = R0 + s * SB + l;
            const int rhi = kind == K_FBND ? fr.f : fr.n;
            if (r < min(Re, rhi)) row_out(kind, fr, r, sum, (T *)nullptr, x);
        }
        __syncthreads();
    }
}

// Warp task: all strips of rows [Rb, Re) of one kind by one warp, its tiles
// double-buffered; lane l accumulates row Rb + 32 s + l of strip s.
// `issued`: the first tile is already in flight.
template <typename T>
__device__ __forceinline__ void warp_rows(int kind, const Front<T> &fr, int Rb, int Re, const T *vec, int vbase, T *buf0, T *buf1,
                          T *out, double *x, bool issued) {
    const int lane = threadIdx.x & 31;
    const int nstr = (Re - Rb + SB - 1) / SB;
    const int rhi = min(Re, kind == K_FBND ? fr.f : fr.n);
    Cursor cur{kind, fr.n, fr.f, Rb, nstr, 0, 0};
    int si = 0, ti = 0;
    bool have = cur.locate(0, si, ti);
    if (have && !issued) issue_item(kind, fr.n, fr.f, Rb, si, ti, fr.F, buf0, lane);
    T acc = T(0);
    int cs = 0;
    for (int it = 0; have; ++it) {
        for (; cs < si; ++cs) {
            const int r = Rb + cs * SB + lane;
            if (r < rhi) row_out(kind, fr, r, acc, out, x);
            acc = T(0);
        }
        int sn = 0, tn = 0;
        const bool more = cur.locate(it + 1, sn, tn);
        if (more) {
            issue_item(kind, fr.n, fr.f, Rb, sn, tn, fr.F, (it & 1) ? buf0 : buf1, lane);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncwarp();
        const T *b = (it & 1) ? buf1 : buf0;
        const Strip g = strip_of(kind, fr.n, fr.f, Rb + si * SB);
        const T *v = vec + (g.c0 + ti * SB - vbase);
        acc += ti == g.diag ? tile_dot_tri(b, v, lane, kind == K_FOWN) : tile_dot(b, v, lane);
        __syncwarp();
        have = more;
        si = sn;
        ti = tn;
    }
    for (; cs < nstr; ++cs) {
        const int r = Rb + cs * SB + lane;
        if (r < rhi) row_out(kind, fr, r, acc, out, x);
        acc = T(0);
    }
}

// Bounded wait of one thread; on giving up it raises the abort and error words.
__device__ __forceinline__ void task_wait(FlowHeader *H, const int *ctr, int wait, int target) {
    if (wait >= 0 && !flow_wait(ctr + wait, target, &H->abort)) {
        atomicExch(&H->abort, 1);
        atomicExch(&H->err, TF_ERR_TIMEOUT);
    }
    __threadfence();
}

// One small front's whole sweep by one warp (bundle tasks).
template <typename T>
__device__ __forceinline__ void warp_front(bool fwd, const Front<T> &fr, const NodeFlow &nf, FlowHeader *H, int *ctr, T *buf0,
                           T *buf1, T *va, T *vb, double *x) {
    const int lane = threadIdx.x & 31;
    const int n = fr.n, f = fr.f;
    const int k1 = fwd ? K_FOWN : K_BBND;
    // the first tile does not depend on the wait
    {
        Cursor cur{k1, n, f, 0, (n + SB - 1) / SB, 0, 0};
        int si, ti;
        if (cur.locate(0, si, ti)) issue_item(k1, n, f, 0, si, ti, fr.F, buf0, lane);
    }
    if (lane == 0) task_wait(H, ctr, fwd ? nf.fw_wait : nf.bw_wait, fwd ? nf.fw_target : nf.bw_target);
    __syncwarp();
    const int padn = (n + SB - 1) / SB * SB;
    for (int c = n + lane; c < padn; c += 32) vb[c] = T(0);
    if (fwd) {
        for (int c = lane; c < padn; c += 32) va[c] = c < n ? (T)__ldcg(x + fr.g[fr.pv[c]]) : T(0);
        __syncwarp();
        warp_rows(K_FOWN, fr, 0, n, va, 0, buf0, buf1, vb, x, true);
        __syncwarp();
        warp_rows(K_FBND, fr, n, f, vb, 0, buf0, buf1, (T *)nullptr, x, false);
    } else {
        const int len = f - n, pad = (len + SB - 1) / SB * SB;
        for (int c = lane; c < pad; c += 32) va[c] = c < len ? (T)__ldcg(x + fr.g[n + c]) : T(0);
        __syncwarp();
        warp_rows(K_BBND, fr, 0, n, va, n, buf0, buf1, vb, x, true);
        __syncwarp();
        warp_rows(K_BOWN, fr, 0, n, vb, 0, buf0, buf1, (T *)nullptr, x, false);
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) atomicAdd(ctr + (fwd ? nf.fw_signal : nf.bw_signal), 1);
}

template <typename T>
__global__ void __launch_bounds__(FTHREADS, 1) flow_kernel(DevPlan P, const T *fronts, const int32_t *piv, double *x,
                                                        char *work) {
    extern __shared__ unsigned char smem_raw[];
    T *tiles = reinterpret_cast<T *>(smem_raw);   // [FW][2] tiles
    T *red = tiles + 2 * FW * TILE;                // [FW][FSPT][32]
    T *vec = red + FW * FSPT * SB;                 // CTA tasks: [vlen]; bundles: [FW][2][FUSE_F]
    FlowHeader *H = reinterpret_cast<FlowHeader *>(work);
    int *ctr = reinterpret_cast<int *>(work + sizeof(FlowHeader));
    const int ntasks = H->ntasks;
    const FlowTask *tasks = reinterpret_cast<const FlowTask *>(work + H->tasks_off);
    const NodeFlow *nodes = reinterpret_cast<const NodeFlow *>(work + H->nodes_off);
    double *ybuf = reinterpret_cast<double *>(work + H->ybuf_off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ int s_ticket;
    for (;;) {
        if (threadIdx.x == 0) s_ticket = atomicAdd(&H->ticket, 1);
        __syncthreads();
        const int ti = s_ticket;
        if (ti >= ntasks) break;
        const FlowTask tk = tasks[ti];
        if (tk.kind == K_WFWD || tk.kind == K_WBWD) {
            // a bundle of up to FW small fronts of one height, one per warp
            if (warp < tk.r0) {
                const int node = tk.node + warp;
                const Front<T> fr = front_of(P, node, fronts, piv, ybuf);
                T *b0 = tiles + (2 * warp) * TILE;
                T *va = vec + (2 * warp) * FUSE_F;
                warp_front(tk.kind == K_WFWD, fr, nodes[node], H, ctr, b0, b0 + TILE, va, va + FUSE_F, x);
            }
            __syncthreads();
            continue;
        }
        const Front<T> fr = front_of(P, tk.node, fronts, piv, ybuf);
        const int n = fr.n, f = fr.f;
        const int kind = tk.kind, Rb = tk.r0, Re = tk.r1;
        products_prefetch(kind, n, f, Rb, min(FSPT, (Re - Rb + SB - 1) / SB), fr.F, tiles);
        if (threadIdx.x == 0) task_wait(H, ctr, tk.wait, tk.target);
        __syncthreads();
        // the task's vector, zero past its end up to the next tile
        int vbase = 0;
        if (kind == K_FOWN) {
            const int pad = (Re + SB - 1) / SB * SB;
            for (int c = threadIdx.x; c < pad; c += FTHREADS)
                vec[c] = c < Re ? (T)__ldcg(x + fr.g[fr.pv[c]]) : T(0);
        } else if (kind == K_FBND) {
            const int pad = (n + SB - 1) / SB * SB;
            for (int c = threadIdx.x; c < pad; c += FTHREADS) vec[c] = c < n ? (T)__ldcg(fr.y + c) : T(0);
        } else if (kind == K_BBND) {
            const int len = f - n, pad = (len + SB - 1) / SB * SB;
            vbase = n;
            for (int c = threadIdx.x; c < pad; c += FTHREADS) vec[c] = c < len ? (T)__ldcg(x + fr.g[n + c]) : T(0);
        } else {
            const int pad = (n + SB - 1) / SB * SB;
            for (int c = Rb + threadIdx.x; c < pad; c += FTHREADS) vec[c] = c < n ? (T)__ldcg(fr.y + c) : T(0);
        }
        __syncthreads();
        run_rows(kind, fr, Rb, Re, vec, vbase, tiles, red, x, true);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0 && tk.signal >= 0) atomicAdd(ctr + tk.signal, 1);
        (void)lane;
    }
}

// ---------------------------------------------------------------------------
// Host side: the task list.
// ---------------------------------------------------------------------------
struct FlowPlanHost {
    std::vector<int32_t> n, f, parent;
    int64_t idx_total = 0;
};

static int flow_read_plan(const tf_nd_plan *p, FlowPlanHost &h) {
    const int nn = p->nnodes;
    h.n.resize(nn);
    h.f.resize(nn);
    h.parent.resize(nn);
    if (cudaMemcpy(h.n.data(), p->d_n_own, nn * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h.f.data(), p->d_f, nn * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h.parent.data(), p->d_parent, nn * sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&h.idx_total, p->d_idx_off + nn, sizeof(int64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return TF_ERR_CUDA;
    return TF_OK;
}

static int64_t strip_tiles(int kind, int n, int f, int R) {
    const int nb = (f - n + SB - 1) / SB, no = (n + SB - 1) / SB;
    if (kind == K_FOWN) return R / SB + 1;
    if (kind == K_FBND) return no;
    if (kind == K_BBND) return nb;
    return (n - R + SB - 1) / SB;
}

// Row ranges [r0, r1) of the tasks of one kind: consecutive strips until
// `chunk` tiles or FSPT strips.  A kind without tiles (a front with no
// boundary, backward) still gets its tasks: they copy y to t.
static void chunks(int kind, int n, int f, int chunk, std::vector<std::pair<int, int>> &out) {
    out.clear();
    const int lo = kind == K_FBND ? n : 0, hi = kind == K_FBND ? f : n;
    int r0 = lo, ns = 0;
    int64_t tiles = 0;
    for (int R = lo; R < hi; R += SB) {
        tiles += strip_tiles(kind, n, f, R);
        ++ns;
        if (ns == FSPT || tiles >= chunk || R + SB >= hi) {
            out.emplace_back(r0, std::min(R + SB, hi));
            r0 = R + SB;
            ns = 0;
            tiles = 0;
        }
    }
}

static int flow_build(const tf_nd_plan *p, const FlowPlanHost &h, int fuse_tiles, int chunk_tiles,
                      std::vector<FlowTask> &tasks, std::vector<NodeFlow> &nodes) {
    const int nn = p->nnodes;
    if (chunk_tiles < 1) chunk_tiles = 1;
    std::vector<int> ep(nn, -1);
    for (int i = 0; i < nn; ++i) {
        if (h.n[i] < 0 || h.f[i] < h.n[i]) return TF_ERR_ARG;
        int a = h.parent[i];
        while (a >= 0 && h.n[a] == 0) a = h.parent[a];
        ep[i] = a;
        if (h.n[i] > 0 && h.f[i] > h.n[i] && a < 0) return TF_ERR_ARG;   // boundary rows need an ancestor
    }
    // small fronts go to warp tasks; the others are split into CTA tasks
    std::vector<char> fused(nn, 0);
    std::vector<std::vector<std::pair<int, int>>> ch(4 * (size_t)nn);   // per front: FOWN, FBND, BBND, BOWN
    const int kinds[4] = {K_FOWN, K_FBND, K_BBND, K_BOWN};
    for (int i = 0; i < nn; ++i) {
        const int n = h.n[i], f = h.f[i];
        if (n == 0) continue;
        const int64_t no = (n + SB - 1) / SB, nb = (f - n + SB - 1) / SB;
        const int64_t sweep = no * (no + 1) / 2 + no * nb;
        fused[i] = fuse_tiles > 0 && sweep <= fuse_tiles && f <= FUSE_F;
        if (fused[i]) continue;
        for (int k = 0; k < 4; ++k) chunks(kinds[k], n, f, chunk_tiles, ch[4 * (size_t)i + k]);
    }
    // tasks finishing each sweep of a front; forward targets of the parents
    auto nfwd_fin = [&](int i) -> int {
        if (fused[i]) return 1;
        return (int)(h.f[i] > h.n[i] ? ch[4 * (size_t)i + 1].size() : ch[4 * (size_t)i].size());
    };
    auto nbwd_fin = [&](int i) -> int { return fused[i] ? 1 : (int)ch[4 * (size_t)i + 3].size(); };
    std::vector<int> kids(nn, 0);
    for (int i = 0; i < nn; ++i)
        if (h.n[i] > 0 && h.f[i] > h.n[i]) kids[ep[i]] += nfwd_fin(i);
    // the counters of a front: forward waits for its children, backward for
    // its parent (without boundary: for its own forward)
    nodes.assign(nn, NodeFlow{});
    for (int i = 0; i < nn; ++i) {
        NodeFlow &nf = nodes[i];
        const bool bnd = h.f[i] > h.n[i];
        nf.fw_target = kids[i];
        nf.fw_wait = kids[i] > 0 ? 4 * i + C_KIDS : -1;
        nf.fw_signal = bnd ? 4 * ep[i] + C_KIDS : 4 * i + C_FA;
        nf.bw_wait = bnd ? 4 * ep[i] + C_BWD : 4 * i + C_FA;
        nf.bw_target = h.n[i] == 0 ? 0 : bnd ? nbwd_fin(ep[i]) : nfwd_fin(i);
        nf.bw_signal = 4 * i + C_BWD;
    }
    tasks.clear();
    auto push = [&](int node, int kind, int r0, int r1, int wait, int target, int signal) {
        FlowTask t;
        t.node = node; t.kind = kind; t.r0 = r0; t.r1 = r1;
        t.wait = target > 0 ? wait : -1; t.target = target; t.signal = signal; t.pad = 0;
        tasks.push_back(t);
    };
    // consecutive small fronts of one height, at most FW per bundle
    auto bundles = [&](int a, int b, int kind) {
        for (int i = a; i < b;) {
            if (h.n[i] == 0 || !fused[i]) { ++i; continue; }
            int j = i;
            while (j < b && j - i < FW && h.n[j] > 0 && fused[j]) ++j;
            push(i, kind, j - i, 0, -1, 0, -1);
            i = j;
        }
    };
    // forward, leaves first; per height the bundles, the own-row tasks of the
    // split fronts, then their boundary tasks
    for (int lv = 0; lv < p->nlevels; ++lv) {
        const int a = p->level_ptr[lv], b = p->level_ptr[lv + 1];
        bundles(a, b, K_WFWD);
        for (int i = a; i < b; ++i) {
            if (h.n[i] == 0 || fused[i]) continue;
            for (auto &c : ch[4 * (size_t)i])
                push(i, K_FOWN, c.first, c.second, nodes[i].fw_wait, nodes[i].fw_target, 4 * i + C_FA);
        }
        for (int i = a; i < b; ++i) {
            if (h.n[i] == 0 || fused[i]) continue;
            const int nfa = (int)ch[4 * (size_t)i].size();
            for (auto &c : ch[4 * (size_t)i + 1])
                push(i, K_FBND, c.first, c.second, 4 * i + C_FA, nfa, 4 * ep[i] + C_KIDS);
        }
    }
    // backward, root first
    for (int lv = p->nlevels - 1; lv >= 0; --lv) {
        const int a = p->level_ptr[lv], b = p->level_ptr[lv + 1];
        for (int i = a; i < b; ++i) {
            if (h.n[i] == 0 || fused[i]) continue;
            for (auto &c : ch[4 * (size_t)i + 2])
                push(i, K_BBND, c.first, c.second, nodes[i].bw_wait, nodes[i].bw_target, 4 * i + C_BA);
        }
        for (int i = a; i < b; ++i) {
            if (h.n[i] == 0 || fused[i]) continue;
            const int nba = (int)ch[4 * (size_t)i + 2].size();
            for (auto &c : ch[4 * (size_t)i + 3]) push(i, K_BOWN, c.first, c.second, 4 * i + C_BA, nba, 4 * i + C_BWD);
        }
        bundles(a, b, K_WBWD);
    }
    return TF_OK;
}

static size_t align16(size_t b) { return (b + 15) / 16 * 16; }

struct FlowLayout {
    size_t ctr_off, ybuf_off, nodes_off, tasks_off, total;
};

static FlowLayout flow_layout(int nnodes, int64_t idx_total, size_t ntasks) {
    FlowLayout L;
    L.ctr_off = sizeof(FlowHeader);
    L.ybuf_off = align16(L.ctr_off + 16 * (size_t)nnodes);
    L.nodes_off = align16(L.ybuf_off + 8 * (size_t)idx_total);
    L.tasks_off = align16(L.nodes_off + sizeof(NodeFlow) * (size_t)nnodes);
    L.total = L.tasks_off + sizeof(FlowTask) * ntasks;
    return L;
}

// Shared memory: the warps' tile buffers, the CTA tasks' partial sums, and a
// vector area holding a CTA task's vector (the widest front) or the bundles'
// two vectors per warp.
template <typename T>
static size_t flow_smem(const tf_nd_plan *p) {
    int m = 0;
    for (int h = 0; h < p->nlevels; ++h) m = std::max(m, p->max_f[h]);
    const size_t vlen = std::max((size_t)(m + SB - 1) / SB * SB, (size_t)2 * FW * FUSE_F);
    return sizeof(T) * ((size_t)2 * FW * TILE + (size_t)FW * FSPT * SB + vlen);
}

template <typename T>
static int solve_flow(const tf_nd_plan *p, const T *fronts, const int32_t *piv, double *x, void *work,
                      cudaStream_t s) {
    int e = check_plan(p);
    if (e) return e;
    if (!fronts || !piv || !x || !work) return TF_ERR_ARG;
    const size_t smem = flow_smem<T>(p);
    if ((e = ensure_smem((const void *)flow_kernel<T>, smem))) return e;
    int dev = 0, nsm = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, flow_kernel<T>, FTHREADS, smem) != cudaSuccess)
        return TF_ERR_CUDA;
    if (occ < 1) return TF_ERR_SIZE;
    char *w = static_cast<char *>(work);
    if (cudaMemsetAsync(w + FLOW_RESET_OFF, 0, sizeof(FlowHeader) - FLOW_RESET_OFF + 16 * (size_t)p->nnodes, s) !=
        cudaSuccess)
        return TF_ERR_CUDA;
    const DevPlan D = dev_plan(p, p->d_rank);
    flow_kernel<T><<<nsm * occ, FTHREADS, smem, s>>>(D, fronts, piv, x, w);
    launched();
    return cuda_status();
}

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" size_t tf_nd_flow_workspace_bytes(const tf_nd_plan *plan, int fuse_tiles, int chunk_tiles) {
    if (nd::check_plan(plan)) return 0;
    nd::FlowPlanHost h;
    if (nd::flow_read_plan(plan, h)) return 0;
    std::vector<nd::FlowTask> tasks;
    std::vector<nd::NodeFlow> nodes;
    if (nd::flow_build(plan, h, fuse_tiles, chunk_tiles, tasks, nodes)) return 0;
    return nd::flow_layout(plan->nnodes, h.idx_total, tasks.size()).total;
}

extern "C" int tf_nd_flow_prepare(const tf_nd_plan *plan, void *d_work, size_t work_bytes, int elem_size,
                                  int fuse_tiles, int chunk_tiles) {
    int e = nd::check_plan(plan);
    if (e) return e;
    if (!d_work || (elem_size != 4 && elem_size != 8)) return TF_ERR_ARG;
    // the launch needs its shared memory: refuse here rather than at the first solve
    e = elem_size == 8 ? nd::ensure_smem((const void *)nd::flow_kernel<double>, nd::flow_smem<double>(plan))
                       : nd::ensure_smem((const void *)nd::flow_kernel<float>, nd::flow_smem<float>(plan));
    if (e) return e;
    nd::FlowPlanHost h;
    if ((e = nd::flow_read_plan(plan, h))) return e;
    std::vector<nd::FlowTask> tasks;
    std::vector<nd::NodeFlow> nodes;
    if ((e = nd::flow_build(plan, h, fuse_tiles, chunk_tiles, tasks, nodes))) return e;
    const nd::FlowLayout L = nd::flow_layout(plan->nnodes, h.idx_total, tasks.size());
    if (work_bytes < L.total) return TF_ERR_SIZE;
    nd::FlowHeader hd = {};
    hd.ntasks = (int32_t)tasks.size();
    hd.tasks_off = (int64_t)L.tasks_off;
    hd.ybuf_off = (int64_t)L.ybuf_off;
    hd.nodes_off = (int64_t)L.nodes_off;
    char *w = static_cast<char *>(d_work);
    if (cudaMemcpy(w, &hd, sizeof(hd), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(w + L.ctr_off, 0, L.ybuf_off - L.ctr_off) != cudaSuccess ||
        cudaMemcpy(w + L.nodes_off, nodes.data(), sizeof(nd::NodeFlow) * nodes.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(w + L.tasks_off, tasks.data(), sizeof(nd::FlowTask) * tasks.size(), cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return TF_ERR_CUDA;
    return TF_OK;
}

extern "C" int tf_nd_flow_tasks_host(int nnodes, const int32_t *n_own, const int32_t *f, const int32_t *parent,
                                     int nlevels, const int32_t *level_ptr, int fuse_tiles, int chunk_tiles,
                                     int32_t *tasks, int32_t *nodes, int max_tasks, int *ntasks) {
    if (nnodes <= 0 || nlevels <= 0 || !n_own || !f || !parent || !level_ptr || !ntasks) return TF_ERR_ARG;
    nd::FlowPlanHost h;
    h.n.assign(n_own, n_own + nnodes);
    h.f.assign(f, f + nnodes);
    h.parent.assign(parent, parent + nnodes);
    tf_nd_plan p = {};
    p.nnodes = nnodes;
    p.nlevels = nlevels;
    p.level_ptr = level_ptr;
    std::vector<nd::FlowTask> t;
    std::vector<nd::NodeFlow> nf;
    const int e = nd::flow_build(&p, h, fuse_tiles, chunk_tiles, t, nf);
    if (e) return e;
    *ntasks = (int)t.size();
    if (!tasks || !nodes) return TF_OK;          // size query
    if ((int)t.size() > max_tasks) return TF_ERR_SIZE;
    std::copy_n(reinterpret_cast<const int32_t *>(t.data()), 8 * t.size(), tasks);
    std::copy_n(reinterpret_cast<const int32_t *>(nf.data()), 8 * nf.size(), nodes);
    return TF_OK;
}

extern "C" int tf_nd_solve_flow_f64(const tf_nd_plan *plan, const double *d_fronts, const int32_t *d_piv, double *d_x,
                                    void *d_work, tf_stream_t stream) {
    return nd::solve_flow<double>(plan, d_fronts, d_piv, d_x, d_work, (cudaStream_t)stream);
}

extern "C" int tf_nd_solve_flow_f32(const tf_nd_plan *plan, const float *d_fronts, const int32_t *d_piv, double *d_x,
                                    void *d_work, tf_stream_t stream) {
    return nd::solve_flow<float>(plan, d_fronts, d_piv, d_x, d_work, (cudaStream_t)stream);
}

extern "C" int tf_nd_flow_status(void *d_work) {
    if (!d_work) return TF_ERR_ARG;
    int32_t err = 0;
    if (cudaMemcpy(&err, d_work, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess) return TF_ERR_CUDA;
    if (err != 0 && cudaMemset(d_work, 0, sizeof(err)) != cudaSuccess) return TF_ERR_CUDA;
    return err;
}
