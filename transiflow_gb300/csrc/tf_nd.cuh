// Declarations shared by the two translation units of the nested-dissection
// multifrontal LU: tf_nd.cu (fronts, trailing updates, extend-add, the
// solves and the C ABI) and tf_nd_panel.cu (the panel factorisations, the
// longest part of the build, compiled in parallel with the rest).
#pragma once

#include "tf_common.cuh"

#include <cooperative_groups.h>

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

// Opts a kernel in to `bytes` of dynamic shared memory on the current device
// (TF_ERR_SIZE when static plus dynamic shared memory would not fit).
int ensure_smem(const void *kernel, size_t bytes);

DevPlan dev_plan(const tf_nd_plan *p, const int32_t *rank);
int check_plan(const tf_nd_plan *p);

// x[bnd] -= L21 y (FWD) or x[own] -= U12 x[bnd] for every front of one tree
// height (rows x cols at most per front).
template <typename T, bool FWD>
void bnd(const DevPlan &D, int node0, int cnt, int rows, int cols, const T *fronts, double *x, cudaStream_t s);

// Pivoted LU of the 32-column panel at column k of every front of one tree
// height (node0 .. node0+cnt-1, at most `rows` panel rows), including the
// row swaps of the columns outside the panel.
template <typename T>
int panel(const DevPlan &D, int node0, int cnt, int k, int rows, int nsm, T *fronts, int32_t *piv, int32_t *info,
          cudaStream_t s);

}  // namespace nd
}  // namespace tf
