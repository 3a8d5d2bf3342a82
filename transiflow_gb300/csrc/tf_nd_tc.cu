// Tensor-core trailing updates of the FP32 multifrontal LU (tcgen05, TF32).
//
// The FP32 factorisation is blocked in two levels (tf_nd.cu, factor<float>):
// inside an outer block of KB = 256 own columns the 32-column panels update
// only the block's own columns; once the block is factored (and its block row
// solved), every front of the tree height receives one rank-w update (w <= KB)
//     F[r][j] -= sum_{q < w} L[r][K0 + q] U[K0 + q][j],   r, j >= E = K0 + w,
// which is this kernel.  One CTA computes a 128 x 256 tile of the product
// on the tensor cores: K runs in chunks of 32 (one 128-byte swizzle row of
// FP32), both operands are staged K-major in shared memory with the 128-byte
// swizzle (A = L rows, B = U columns transposed while staging, so both are
// read from global memory in 32-byte sectors and written to shared memory
// without bank conflicts), and one thread issues the tcgen05.mma
// instructions that accumulate in FP32 in tensor memory (128 lanes x 256
// columns).  Operands are rounded to TF32 (round to nearest); with TERMS = 3
// each is also split into a TF32 high part and a TF32 remainder and the
// product is a_hi b_hi + a_hi b_lo + a_lo b_hi (three MMAs per step), which
// keeps the factors close to FP32 quality (plain TF32 products tripled the
// GMRES iterations of the preconditioned solves in the tests).  The
// epilogue (tcgen05.ld -> shared memory -> coalesced read-modify-write of the
// front) is bound by HBM, so the extra MMAs cost little.
//
// Fronts are row-major with arbitrary row length f, so rows start at any
// 4-byte alignment: plain 4-byte loads, no TMA.
//
// Every mbarrier wait is bounded; a wait that gives up increments the
// factorisation's info counter (the solve is then reported as failed), the
// CTA skips its epilogue, waits once more (bounded) for its MMAs and frees
// its tensor memory.

#include "tf_nd.cuh"
#include "tf_tcgen05.cuh"

namespace tf {
namespace nd {

constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
constexpr int TC_THREADS = 256;
// two CTAs per SM, so that one CTA's tensor-core work overlaps the other's
// gather and epilogue: one stage with split operands (96 KB), two without
template <int TERMS>
struct TcStages {
    static constexpr int n = TERMS == 1 ? 2 : 1;
};
constexpr int TC_A_BYTES = TC_BM * 128;                      // 128 rows x 32 FP32
constexpr int TC_B_BYTES = TC_BN * 128;                      // 256 rows x 32 FP32
constexpr int TC_EPI_COLS = 128;                             // epilogue pass width
constexpr int TC_EPI_STRIDE = TC_EPI_COLS + 4;               // floats, conflict-free
// a stage holds A and B (TERMS = 1) or their high parts and remainders
template <int TERMS>
struct TcSizes {
    static constexpr int stage = (TERMS == 1 ? 1 : 2) * (TC_A_BYTES + TC_B_BYTES);
    static constexpr size_t smem = (size_t)TcStages<TERMS>::n * stage + 1024;   // + alignment slack
    static_assert(TC_BM * TC_EPI_STRIDE * 4 <= TcStages<TERMS>::n * stage, "epilogue staging must fit");
};

// Instruction descriptor of tcgen05.mma .kind::tf32: D FP32 (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                              ((uint32_t)(TC_BM >> 4) << 24);

using namespace tc5;

// Byte offset of FP32 element (row, q), q < 32, in a 128-byte-swizzled
// K-major tile whose base is 1024-byte aligned.
__device__ __forceinline__ unsigned sw128_off(int row, int q) { return sw128_piece(row, q >> 2) + (q & 3) * 4; }

__device__ __forceinline__ uint32_t to_tf32(float v) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(v));
    return r;
}

__device__ __forceinline__ void tc_mma(unsigned tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
    asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)acc) : "memory");
}

template <int TERMS>
__global__ void __launch_bounds__(TC_THREADS, 2)
    tc_update_kernel(DevPlan P, int node0, int K0, float *fronts, int32_t *info) {
    constexpr int STAGE = TcSizes<TERMS>::stage;
    constexpr int TC_STAGES = TcStages<TERMS>::n;
    extern __shared__ unsigned char tc_raw[];
    __shared__ __align__(8) uint64_t bar[3];
    __shared__ unsigned tmem_slot;
    const int node = node0 + blockIdx.z;
    const int n = P.n_own[node], f = P.f[node];
    const int E = min(K0 + KB, n);
    const int w = E - K0;
    const int r0 = E + blockIdx.y * TC_BM, c0 = E + blockIdx.x * TC_BN;
    // uniform over the CTA, before any barrier or allocation
    if (w <= 0 || r0 >= f || c0 >= f) return;
    float *F = fronts + P.front_off[node];
    unsigned char *smem = reinterpret_cast<unsigned char *>(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    const unsigned sbase = smem_addr(smem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int s = 0; s <= TC_STAGES; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&bar[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     ::"r"(smem_addr(&tmem_slot)), "r"((unsigned)TC_BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const unsigned tmem = tmem_slot;

    bool ok = true;
    const int nk = (w + 31) / 32;
    for (int c = 0; c < nk; ++c) {
        const int s = c % TC_STAGES;
        const unsigned As = sbase + s * STAGE, Bs = As + TC_A_BYTES;
        // remainders (TERMS = 3) after the high parts
        const unsigned Al = Bs + TC_B_BYTES, Bl = Al + TC_A_BYTES;
        const int qc = 32 * c;
        // gather first (all loads in flight), then the swizzled stores
        float va[TC_BM / 8], vb[32];
        {
            const bool qok = qc + lane < w;
            const float *src = F + (size_t)K0 + qc + lane;
#pragma unroll
            for (int i = 0; i < TC_BM / 8; ++i) {
                const int r = r0 + warp * (TC_BM / 8) + i;
                va[i] = (qok && r < f) ? src[(size_t)r * f] : 0.f;
            }
        }
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const int q = (t & 7) * 4 + (lane & 3);
            const int j = (warp * 4 + (t >> 3)) * 8 + (lane >> 2);
            const int cj = c0 + j;
            vb[t] = (qc + q < w && cj < f) ? F[(size_t)(K0 + qc + q) * f + cj] : 0.f;
        }
        // the stage is free once the MMAs of chunk c - TC_STAGES are done
        // (waited for after this chunk's loads are in flight)
        if (c >= TC_STAGES && !wait_parity(&bar[s], (unsigned)((c / TC_STAGES - 1) & 1))) ok = false;
#pragma unroll
        for (int i = 0; i < TC_BM / 8; ++i) {
            const int row = warp * (TC_BM / 8) + i;
            const uint32_t hi = to_tf32(va[i]);
            sts_u32(As + sw128_off(row, lane), hi);
            if (TERMS == 3) sts_u32(Al + sw128_off(row, lane), to_tf32(va[i] - __uint_as_float(hi)));
        }
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const int q = (t & 7) * 4 + (lane & 3);
            const int j = (warp * 4 + (t >> 3)) * 8 + (lane >> 2);
            const uint32_t hi = to_tf32(vb[t]);
            sts_u32(Bs + sw128_off(j, q), hi);
            if (TERMS == 3) sts_u32(Bl + sw128_off(j, q), to_tf32(vb[t] - __uint_as_float(hi)));
        }
        // generic-proxy stores visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                if (TERMS == 3) {
                    tc_mma(tmem, sw128_desc(Al + kk * 32), sw128_desc(Bs + kk * 32), TC_IDESC, (c | kk) != 0);
                    tc_mma(tmem, sw128_desc(As + kk * 32), sw128_desc(Bl + kk * 32), TC_IDESC, true);
                    tc_mma(tmem, sw128_desc(As + kk * 32), sw128_desc(Bs + kk * 32), TC_IDESC, true);
                } else {
                    tc_mma(tmem, sw128_desc(As + kk * 32), sw128_desc(Bs + kk * 32), TC_IDESC, (c | kk) != 0);
                }
            }
            commit(&bar[s]);
        }
    }
    if (tid == 0) commit(&bar[TC_STAGES]);
    if (!wait_parity(&bar[TC_STAGES], 0u)) {
        ok = false;
        wait_parity(&bar[TC_STAGES], 0u);
    }
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    ok = __syncthreads_and(ok);

    if (ok) {
        // epilogue in two passes of 128 columns: tensor memory -> shared
        // memory (row per thread) -> read-modify-write of the front rows
        // (a warp per 32 consecutive columns)
        float *Cs = reinterpret_cast<float *>(smem);
        const int lg = warp & 3;               // tensor-memory lanes 32 lg .. 32 lg + 31
        const int row = lg * 32 + lane;
        for (int pass = 0; pass < TC_BN / TC_EPI_COLS; ++pass) {
            if (c0 + pass * TC_EPI_COLS >= f) break;     // uniform
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int col = (warp >> 2) * 64 + h * 32;   // within the pass
                float v[32];
                tmem_ld32(tmem + ((unsigned)(lg * 32) << 16) + (unsigned)(pass * TC_EPI_COLS + col), v);
#pragma unroll
                for (int i = 0; i < 32; i += 4)
                    *reinterpret_cast<float4 *>(Cs + row * TC_EPI_STRIDE + col + i) =
                        make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            }
            __syncthreads();
            // 32 rows per batch: all loads of a batch in flight before its
            // stores (a warp covers 32 consecutive columns of one row)
            const int cl = tid & (TC_EPI_COLS - 1);
            const int cj = c0 + pass * TC_EPI_COLS + cl;
            constexpr int RSTEP = TC_THREADS / TC_EPI_COLS;
            constexpr int BATCH = 32;
            if (cj < f) {
                float *col = F + cj;
#pragma unroll 1
                for (int rb = tid / TC_EPI_COLS; rb < TC_BM; rb += RSTEP * BATCH) {
                    float cur[BATCH];
#pragma unroll
                    for (int u = 0; u < BATCH; ++u) {
                        const int r = r0 + rb + u * RSTEP;
                        cur[u] = (rb + u * RSTEP < TC_BM && r < f) ? col[(size_t)r * f] : 0.f;
                    }
#pragma unroll
                    for (int u = 0; u < BATCH; ++u) {
                        const int rr = rb + u * RSTEP, r = r0 + rr;
                        if (rr < TC_BM && r < f) col[(size_t)r * f] = cur[u] - Cs[rr * TC_EPI_STRIDE + cl];
                    }
                }
            }
            __syncthreads();
        }
    } else if (tid == 0 && info) {
        atomicAdd(info, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"((unsigned)TC_BN)
                     : "memory");
    }
}

template <int TERMS>
static int tc_launch(const DevPlan &D, int node0, int cnt, int K0, int rest, float *fronts, int32_t *info,
                     cudaStream_t s) {
    const int e = ensure_smem((const void *)tc_update_kernel<TERMS>, TcSizes<TERMS>::smem);
    if (e) return e;
    dim3 grid((rest + TC_BN - 1) / TC_BN, (rest + TC_BM - 1) / TC_BM, cnt);
    tc_update_kernel<TERMS><<<grid, TC_THREADS, TcSizes<TERMS>::smem, s>>>(D, node0, K0, fronts, info);
    launched();
    return TF_OK;
}

int tc_update(const DevPlan &D, int node0, int cnt, int K0, int mf, int terms, float *fronts, int32_t *info,
              cudaStream_t s) {
    const int rest = mf - K0;
    if (rest <= 0 || cnt <= 0) return TF_OK;
    if (terms == 1) return tc_launch<1>(D, node0, cnt, K0, rest, fronts, info, s);
    return tc_launch<3>(D, node0, cnt, K0, rest, fronts, info, s);
}

}  // namespace nd
}  // namespace tf

using namespace tf;

extern "C" int tf_nd_tc_update_f32(const tf_nd_plan *plan, int height, int k0, int terms, float *d_fronts,
                                   int32_t *d_info, tf_stream_t stream) {
    if (!plan || !d_fronts || height < 0 || height >= plan->nlevels || k0 < 0 || (terms != 1 && terms != 3))
        return TF_ERR_ARG;
    if (!plan->d_n_own || !plan->d_f || !plan->d_front_off || !plan->level_ptr || !plan->max_f) return TF_ERR_ARG;
    const nd::DevPlan D = nd::dev_plan(plan, plan->d_rank);
    const int node0 = plan->level_ptr[height], cnt = plan->level_ptr[height + 1] - node0;
    const int e = nd::tc_update(D, node0, cnt, k0, plan->max_f[height], terms, d_fronts, d_info,
                                (cudaStream_t)stream);
    return e ? e : cuda_status();
}
