// Shared device helpers for libtfcuda: error mapping, the compile-time
// stencil template and the metric table layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <utility>

#include "../../include/tfcuda.h"

namespace tf {

// Metric table fields, see tf_problem in tfcuda.h.
enum { M_D = 0, M_DP, M_H, M_HP, M_RD, M_RDP, M_RH, M_RHP, M_W0, M_W1 };

// Host-side count of kernel launches issued by the library (tf_launch_count).
extern std::atomic<long long> g_launches;
static inline void launched(long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

static inline int cuda_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TF_OK : TF_ERR_CUDA;
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation may start while the previous kernel of the stream runs;
// pdl_trigger lets the next launch start, pdl_wait blocks until the previous
// kernel has finished and its writes are visible (a no-op without the
// attribute).  Work before pdl_wait may only touch data no earlier launch of
// the sequence writes.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

// Launch with or without programmatic stream serialisation.
template <typename... KArgs, typename... Args>
static inline cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                     cudaStream_t s, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__host__ __device__ constexpr int off_index(int ox, int oy, int oz) { return ox + 3 * oy + 9 * oz; }

// ---------------------------------------------------------------------------
// Stencil template.  Which (d2, offset) an atom row d1 can hold, following the
// primitives of Discretization.py:
//   velocity row a, own velocity : 3/5/7-point star (diffusion + convection)
//   velocity row a, velocity b   : offset_a in {1,2}, offset_b in {0,1}
//                                  (linearised convection u_v_x etc.)
//   velocity row a, pressure     : offset_a in {1,2}   (pressure gradient)
//   velocity row a>=1, T         : offset_a in {1,2}   (buoyancy average)
//   pressure row, velocity b     : offset_b in {0,1}   (divergence)
//   pressure row, pressure       : centre (holds the gauge -1)
//   T row, T                     : star (diffusion + convection)
//   T row, velocity b            : offset_b in {0,1}   (linearised T advection,
//                                  Rayleigh-Benard perturbation term)
//   velocity row a>=1, S; S row   : as for T (salinity: - forward average,
//                                  diffusion + convection, linearised advection)
// Every boundary fold moves offset 0/2 to 1 along its axis inside one
// (d1, d2) pair, and each of these sets is closed under that projection.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr bool in_template(int DIM, int DOF, int d1, int d2, int ox, int oy, int oz) {
    int o[3] = {ox, oy, oz};
    if (DIM == 2 && oz != 1) return false;
    const int P = DIM, T = DIM + 1, S = DIM + 2;
    const bool hasT = DOF > DIM + 1, hasS = DOF > DIM + 2;
    int noncentre = (ox != 1) + (oy != 1) + (oz != 1);
    auto only = [&](int a, int lo, int hi) {
        for (int b = 0; b < 3; ++b) {
            if (b == a) { if (o[b] < lo || o[b] > hi) return false; }
            else if (o[b] != 1) return false;
        }
        return true;
    };
    if (d1 < DIM) {
        const int a = d1;
        if (d2 == d1) return noncentre <= 1;
        if (d2 < DIM) {
            for (int b = 0; b < 3; ++b) {
                if (b == a) { if (o[b] < 1) return false; }
                else if (b == d2) { if (o[b] > 1) return false; }
                else if (o[b] != 1) return false;
            }
            return true;
        }
        if (d2 == P) return only(a, 1, 2);
        if (hasT && d2 == T) return a >= 1 && only(a, 1, 2);
        if (hasS && d2 == S) return a >= 1 && only(a, 1, 2);
        return false;
    }
    if (d1 == P) {
        if (d2 < DIM) return only(d2, 0, 1);
        if (d2 == P) return noncentre == 0;
        return false;
    }
    if ((hasT && d1 == T) || (hasS && d1 == S)) {
        if (d2 == d1) return noncentre <= 1;
        if (d2 < DIM) return only(d2, 0, 1);
        return false;
    }
    return false;
}

// Slot layout of one cell: rows d1 = 0..DOF-1 in order, each row's entries
// sorted by column, i.e. by (oz, oy, ox, d2).
template <int DIM, int DOF>
struct Layout {
    int slot[DOF][DOF][27];   // position inside the cell chunk, -1 if absent
    int rowoff[DOF + 1];
    __host__ __device__ constexpr Layout() : slot{}, rowoff{} {
        int p = 0;
        for (int d1 = 0; d1 < DOF; ++d1) {
            rowoff[d1] = p;
            for (int d2 = 0; d2 < DOF; ++d2)
                for (int o = 0; o < 27; ++o) slot[d1][d2][o] = -1;
            for (int oz = 0; oz < 3; ++oz)
                for (int oy = 0; oy < 3; ++oy)
                    for (int ox = 0; ox < 3; ++ox)
                        for (int d2 = 0; d2 < DOF; ++d2)
                            if (in_template(DIM, DOF, d1, d2, ox, oy, oz))
                                slot[d1][d2][off_index(ox, oy, oz)] = p++;
        }
        rowoff[DOF] = p;
    }
    __host__ __device__ constexpr int width() const { return rowoff[DOF]; }
};

// Dispatch on the (dim, dof) combinations that are compiled in.
#define TF_DISPATCH(dim, dof, CALL)                                   \
    do {                                                              \
        if ((dim) == 2 && (dof) == 3) { CALL(2, 3); }                 \
        else if ((dim) == 2 && (dof) == 4) { CALL(2, 4); }            \
        else if ((dim) == 2 && (dof) == 5) { CALL(2, 5); }            \
        else if ((dim) == 3 && (dof) == 4) { CALL(3, 4); }            \
        else if ((dim) == 3 && (dof) == 5) { CALL(3, 5); }            \
        else return TF_ERR_UNSUPPORTED;                               \
    } while (0)

}  // namespace tf
