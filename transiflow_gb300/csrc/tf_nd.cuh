// Declarations shared by the two translation units of the nested-dissection
// multifrontal LU: tf_nd.cu (fronts, trailing updates, extend-add, the
// solves and the C ABI) and tf_nd_panel.cu (the panel factorisations, the
// longest part of the build, compiled in parallel with the rest).
#pragma once

#include "tf_common.cuh"

#include <cooperative_groups.h>

#include <functional>

namespace tf {
namespace nd {

namespace cg = cooperative_groups;

constexpr int NB = 32;       // panel width
constexpr int TM = 64;       // gemm tile rows
constexpr int TN = 64;       // gemm tile cols
constexpr int THREADS = 256;
// Outer block of the two-level FP32 factorisation: the 32-column panels of a
// block update only the block's columns and rows, the rest of the front gets
// one rank-KB update on the tensor cores per block (tf_nd_tc.cu).
constexpr int KB = 256;
// Region of a SIMT trailing update (gemm kernels in tf_nd.cu), for the panel
// at column k inside the outer block starting at K0, E = min(K0 + KB, n):
//   UPD_ALL   rows and columns [k + nb, f)       (one-level factorisation)
//   UPD_COLS  rows [k + nb, f), columns [k + nb, E)
//   UPD_ROWS  rows [k + nb, E), columns [E, f)
enum { UPD_ALL = 0, UPD_COLS = 1, UPD_ROWS = 2 };

struct DevPlan {
    const int32_t *n_own, *f, *parent, *idx, *ea_map, *rank;
    const int64_t *front_off, *idx_off, *ea_off, *piv_off;
};

template <typename T>
__device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// 32 x 32 tiles of a front staged in shared memory by cp.async (8- or
// 4-byte copies: rows of a front start at arbitrary alignment).
constexpr int SB = 32;
constexpr int TSTRIDE = SB + 1;
constexpr int TILE = SB * TSTRIDE;      // elements of one padded 32 x 32 tile

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

// The same over the first nc <= SB columns only (a front's last, partial
// column tile: the FP64 pipe then does only the useful products).
template <typename T>
__device__ __forceinline__ T tile_dot_n(const T *buf, const T *v, int lane, int nc) {
    if (nc >= SB) return tile_dot(buf, v, lane);
    T s = T(0);
    for (int c = 0; c < nc; ++c) s += buf[lane * TSTRIDE + c] * v[c];
    return s;
}

// Opts a kernel in to `bytes` of dynamic shared memory on the current device
// (TF_ERR_SIZE when static plus dynamic shared memory would not fit).
int ensure_smem(const void *kernel, size_t bytes);

DevPlan dev_plan(const tf_nd_plan *p, const int32_t *rank);
int check_plan(const tf_nd_plan *p);

// Numeric factorisation of every front, height by height on stream s; after
// each height (its fronts factored and their Schur complements added into the
// parents) `after_level(h)`, when given, may enqueue work that depends on it.
template <typename T>
int factor(const tf_nd_plan *p, const double *vals, T *fronts, int32_t *piv, int32_t *info, cudaStream_t s,
           const std::function<int(int)> *after_level);

// Application with the inverted FP64 own blocks (tf_nd_inv.cu), one launch
// pair per height: the forward sweep over heights [0, h_end) or the backward
// sweep over heights h_end-1 .. 0; y / t of the own rows in `packed` (one
// value per front index entry).
template <typename T>
int inv_levels(const tf_nd_plan *p, const DevPlan &D, const T *fronts, const int32_t *piv, double *x, double *packed,
               int h_end, bool fwd, cudaStream_t s);

// x[bnd] -= L21 y (FWD) or x[own] -= U12 x[bnd] for every front of one tree
// height (rows x cols at most per front).
template <typename T, bool FWD>
void bnd(const DevPlan &D, int node0, int cnt, int rows, int cols, const T *fronts, double *x, cudaStream_t s);

// Rank-w tensor-core update F[r][j] -= L[r][K0:E] U[K0:E][j], r, j >= E, of
// every front of one tree height (FP32 fronts, TF32 products -- one term, or
// three for split operands -- with FP32 sums).
int tc_update(const DevPlan &D, int node0, int cnt, int K0, int mf, int terms, float *fronts, int32_t *info,
              cudaStream_t s);

// Pivoted LU of the 32-column panel at column k of every front of one tree
// height (node0 .. node0+cnt-1, at most `rows` panel rows), including the
// row swaps of the columns outside the panel.
template <typename T>
int panel(const DevPlan &D, int node0, int cnt, int k, int rows, int nsm, T *fronts, int32_t *piv, int32_t *info,
          cudaStream_t s);

}  // namespace nd
}  // namespace tf
