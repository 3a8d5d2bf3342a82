// Learned continuation predictor: a stack of 3x3x3 convolutions over the
// cell grid that proposes the correction to the secant predictor of
// pseudo-arclength continuation.  Activations are channels-last
// ([cell][channel], cell = i + nx*(j + ny*k), the ordering of the state
// vector), operands are BF16 and every product is accumulated in FP32 on the
// tensor cores (tcgen05.mma with tensor-memory accumulators).  Training runs here too: the gradient
// with respect to the input of a layer is the same convolution with the
// mirrored, transposed weights; the weight gradient is an FP32 reduction over
// cells written as per-chunk partial sums and reduced in a fixed order, so a
// training run is deterministic; Adam updates FP32 master weights and writes
// both BF16 layouts the convolutions read.
//
// Weight layouts (tap = (ox+1) + 3*(oy+1) + 9*(oz+1), 27 taps):
//   master  w [27][kp][np] FP32, bias [np] FP32
//   forward B [27][np][kp] BF16   (n = output channel, k = input channel)
//   backward-data B [27][kp][np] BF16 holding w[26 - tap], the mirror tap
// Gradients and Adam moments share one layout [28][kp][np]: slot 27 holds the
// bias in its row ci = 0.

#include <cuda_bf16.h>

#include "tf_common.cuh"
#include "tf_tcgen05.cuh"

namespace tf {
namespace sg {

constexpr int WG_CELLS = 1024;    // cells per weight-gradient chunk
constexpr int WG_SUB = 32;        // cells staged in shared memory at a time
constexpr int WG_THREADS = 256;
constexpr int MAX_CH = 32;        // channels per layer, padded to 16 or 32
constexpr int MAX_DOF = 8;

struct FieldScales {
    float a[MAX_DOF];
    float b[MAX_DOF];
};

struct StateScales {
    double a[MAX_DOF];
};

// Neighbour of cell (i, j, k) across tap, or -1 outside the grid (zero padding).
__device__ __forceinline__ int neighbour(int i, int j, int k, int tap, int nx, int ny, int nz) {
    const int a = i + tap % 3 - 1, b = j + (tap / 3) % 3 - 1, c = k + tap / 9 - 1;
    if (a < 0 || a >= nx || b < 0 || b >= ny || c < 0 || c >= nz) return -1;
    return a + nx * (b + ny * c);
}

// One 3x3x3 convolution as an implicit GEMM on the tensor cores: rows (M) are
// 128 consecutive cells per CTA, N the NP output channels, K runs over (tap,
// input channel) in chunks of 64 BF16 values -- one 128-byte swizzle row,
// 64 / KP taps of KP channels (27 taps: 14 chunks at KP = 32, 7 at KP = 16,
// the last one padded with zeros).  The weights of every chunk stay in
// shared memory for the whole CTA (B, K-major: B[tap][n][k] is already K
// contiguous); each chunk of A is gathered by the CTA's 128 threads, one
// cell each (eight 16-byte loads of the neighbour cells' channels, zero
// outside the grid), into one of two swizzled stages while the tensor cores
// work on the other.  One thread issues tcgen05.mma (kind::f16, BF16
// operands, M = 128, N = NP, K = 16 per instruction) accumulating in FP32 in
// tensor memory; the epilogue reads each cell's NP accumulators
// (tcgen05.ld), adds the bias and writes Z (FP32, conv + bias) and A (BF16,
// relu(conv + bias) when relu is set, else conv + bias).  A bounded wait that
// gives up leaves Z and A filled with NaN for the CTA's cells (the training
// loss or the prediction then shows it) instead of hanging.
constexpr int CV_M = 128;          // cells per CTA = tensor-memory lanes
constexpr int CV_THREADS = 128;    // one thread per cell
constexpr int CV_STAGES = 2;

template <int KP, int NP>
struct ConvShape {
    static constexpr int taps = 64 / KP;                        // taps per K chunk
    static constexpr int chunks = (27 + taps - 1) / taps;
    static constexpr int b_chunk = NP * 128;                    // bytes of B per chunk
    static constexpr int b_bytes = chunks * b_chunk;
    static constexpr int a_stage = CV_M * 128;
    static constexpr size_t smem = (size_t)b_bytes + CV_STAGES * a_stage + 1024;
    // kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major,
    // N >> 3 at bit 17, M >> 4 at bit 24
    static constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NP >> 3) << 17) |
                                      ((uint32_t)(CV_M >> 4) << 24);
};

__device__ __forceinline__ void mma_bf16_tc(unsigned tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
    asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)acc) : "memory");
}

template <int KP, int NP>
__global__ void __launch_bounds__(CV_THREADS)
conv_kernel(int nx, int ny, int nz, const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ B,
            const float *__restrict__ bias, float *__restrict__ Z, __nv_bfloat16 *__restrict__ A, int relu) {
    using namespace tc5;
    using S = ConvShape<KP, NP>;
    extern __shared__ unsigned char cv_raw[];
    __shared__ __align__(8) uint64_t bar[CV_STAGES + 1];
    __shared__ unsigned tmem_slot;
    const int ncell = nx * ny * nz;
    const int tid = threadIdx.x, warp = tid >> 5;
    unsigned char *smem = reinterpret_cast<unsigned char *>(((uintptr_t)cv_raw + 1023) & ~(uintptr_t)1023);
    const unsigned sb = smem_addr(smem);          // B, chunk after chunk
    const unsigned sa = sb + S::b_bytes;          // A stages
    if (tid == 0) {
        for (int s = 0; s <= CV_STAGES; ++s) mbar_init1(&bar[s]);
        mbar_init_fence();
    }
    if (warp == 0) tmem_alloc(&tmem_slot, 32);
    // the weights of every chunk: 16-byte piece p of row n of chunk c holds
    // input channels 8p .. 8p + 7 of the chunk's taps
    constexpr int BPIECES = S::chunks * NP * 8;
    for (int q = tid; q < BPIECES; q += CV_THREADS) {
        const int c = q / (NP * 8), rem = q % (NP * 8), n = rem >> 3, p = rem & 7;
        const int tap = c * S::taps + (8 * p) / KP, ci = (8 * p) % KP;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (tap < 27) v = __ldg(reinterpret_cast<const uint4 *>(B + ((size_t)tap * NP + n) * KP + ci));
        sts_v4(sb + c * S::b_chunk + sw128_piece(n, p), v);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = tmem_slot;
    const int cell = blockIdx.x * CV_M + tid;
    const bool valid = cell < ncell;
    const int nxy = nx * ny;
    const int ci0 = valid ? cell % nx : 0, cj0 = valid ? (cell / nx) % ny : 0, ck0 = valid ? cell / nxy : 0;
    bool ok = true;
    for (int c = 0; c < S::chunks; ++c) {
        const int s = c % CV_STAGES;
        const unsigned As = sa + s * S::a_stage;
        uint4 v[8];
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const int tap = c * S::taps + (8 * p) / KP, ch = (8 * p) % KP;
            const int nb = (valid && tap < 27) ? neighbour(ci0, cj0, ck0, tap, nx, ny, nz) : -1;
            v[p] = nb >= 0 ? __ldg(reinterpret_cast<const uint4 *>(X + (size_t)nb * KP + ch))
                           : make_uint4(0u, 0u, 0u, 0u);
        }
        // the stage is free once the MMAs of chunk c - CV_STAGES are done
        if (c >= CV_STAGES && !wait_parity(&bar[s], (unsigned)((c / CV_STAGES - 1) & 1))) ok = false;
#pragma unroll
        for (int p = 0; p < 8; ++p) sts_v4(As + sw128_piece(tid, p), v[p]);
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma_bf16_tc(tmem, sw128_desc(As + kk * 32), sw128_desc(sb + c * S::b_chunk + kk * 32), S::idesc,
                            (c | kk) != 0);
            commit(&bar[s]);
        }
    }
    if (tid == 0) commit(&bar[CV_STAGES]);
    if (!wait_parity(&bar[CV_STAGES], 0u)) {
        ok = false;
        wait_parity(&bar[CV_STAGES], 0u);
    }
    fence_after();
    ok = __syncthreads_and(ok);
    float acc[NP];
    const unsigned taddr = tmem + ((unsigned)(warp * 32) << 16);
    if (NP == 32) tmem_ld32(taddr, acc);
    else tmem_ld16(taddr, acc);
    if (valid) {
        const float qnan = __int_as_float(0x7fc00000);
#pragma unroll
        for (int col = 0; col < NP; col += 4) {
            float z[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) z[u] = ok ? acc[col + u] + (bias ? bias[col + u] : 0.f) : qnan;
            if (Z) *reinterpret_cast<float4 *>(Z + (size_t)cell * NP + col) = make_float4(z[0], z[1], z[2], z[3]);
            if (A) {
                float y[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) y[u] = relu ? fmaxf(z[u], 0.f) : z[u];
                __nv_bfloat162 *ap = reinterpret_cast<__nv_bfloat162 *>(A + (size_t)cell * NP + col);
                ap[0] = __floats2bfloat162_rn(y[0], y[1]);
                ap[1] = __floats2bfloat162_rn(y[2], y[3]);
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_free(tmem, 32);
    }
}

// Partial weight gradient of one chunk of cells and one tap (blockIdx.y; 27 =
// the bias): part[chunk][tap][ci][co] = sum over the chunk's cells c of
// X[c + off(tap)][ci] * dZ[c][co].
__global__ void __launch_bounds__(WG_THREADS)
wgrad_kernel(int nx, int ny, int nz, const __nv_bfloat16 *__restrict__ X, int kp, const float *__restrict__ dZ,
             int np, float *__restrict__ part) {
    __shared__ float xs[WG_SUB][MAX_CH + 1];
    __shared__ float zs[WG_SUB][MAX_CH + 1];
    const int ncell = nx * ny * nz;
    const int tap = blockIdx.y;
    const int c0 = blockIdx.x * WG_CELLS;
    const int c_end = min(c0 + WG_CELLS, ncell);
    const int pairs = kp * np;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int s = c0; s < c_end; s += WG_SUB) {
        for (int e = threadIdx.x; e < WG_SUB * MAX_CH; e += WG_THREADS) {
            const int r = e / MAX_CH, ch = e % MAX_CH;
            const int c = s + r;
            float xv = 0.f, zv = 0.f;
            if (c < c_end) {
                if (ch < np) zv = dZ[(size_t)c * np + ch];
                if (ch < kp) {
                    if (tap == 27) {
                        xv = ch == 0 ? 1.f : 0.f;
                    } else {
                        const int nb = neighbour(c % nx, (c / nx) % ny, c / (nx * ny), tap, nx, ny, nz);
                        if (nb >= 0) xv = __bfloat162float(X[(size_t)nb * kp + ch]);
                    }
                }
            }
            xs[r][ch] = xv;
            zs[r][ch] = zv;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int p = threadIdx.x + q * WG_THREADS;
            if (p < pairs) {
                const int ci = p / np, co = p % np;
                float a = acc[q];
#pragma unroll 8
                for (int r = 0; r < WG_SUB; ++r) a = fmaf(xs[r][ci], zs[r][co], a);
                acc[q] = a;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int p = threadIdx.x + q * WG_THREADS;
        if (p < pairs) part[((size_t)blockIdx.x * 28 + tap) * pairs + p] = acc[q];
    }
}

// out[i] (+)= sum over chunks of part[chunk][i], chunks in order.
__global__ void reduce_kernel(int nchunks, int m, const float *__restrict__ part, float *__restrict__ out,
                              int accumulate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float s = 0.f;
    for (int ch = 0; ch < nchunks; ++ch) s += part[(size_t)ch * m + i];
    out[i] = accumulate ? out[i] + s : s;
}

// Mean-squared loss over the first dof channels of the last layer's output:
// dZ = gscale * (out - tgt) (0 on padded channels), squared errors summed per
// block into part[block].
__global__ void __launch_bounds__(256)
loss_kernel(int ncell, int dof, int np, const float *__restrict__ out, const float *__restrict__ tgt, float gscale,
            float *__restrict__ dzf, __nv_bfloat16 *__restrict__ dzh, double *__restrict__ part) {
    __shared__ double red[256];
    const long long e = (long long)blockIdx.x * 256 + threadIdx.x;
    double sq = 0.0;
    if (e < (long long)ncell * np) {
        const int c = (int)(e / np), ch = (int)(e % np);
        float gr = 0.f;
        if (ch < dof) {
            const float r = out[e] - tgt[(size_t)c * dof + ch];
            sq = (double)r * (double)r;
            gr = gscale * r;
        }
        dzf[e] = gr;
        dzh[e] = __float2bfloat16(gr);
    }
    red[threadIdx.x] = sq;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out[0] = scale * sum of part[0..n), one CTA, fixed order per thread.
__global__ void __launch_bounds__(256) sum_kernel(int n, const double *__restrict__ part, double scale,
                                                  double *__restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = scale * red[0];
}

// dZ = dA where Z > 0, else 0 (the ReLU between layers), in FP32 and BF16.
__global__ void act_grad_kernel(long long n, const float *__restrict__ da, const float *__restrict__ z,
                                float *__restrict__ dzf, __nv_bfloat16 *__restrict__ dzh) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float v = z[e] > 0.f ? da[e] : 0.f;
    dzf[e] = v;
    dzh[e] = __float2bfloat16(v);
}

// Network input: state x and tangent t scaled per variable, then the
// parameter and the step as constant channels, zero padding up to kp.
__global__ void pack_kernel(int ncell, int dof, int kp, const double *__restrict__ x, const double *__restrict__ t,
                            const double *__restrict__ pv, FieldScales sc, FieldScales sp, float mu, float ds,
                            __nv_bfloat16 *__restrict__ X0) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncell * kp) return;
    const long long c = e / kp;
    const int ch = (int)(e % kp);
    const int nf = pv ? 3 : 2;          // fields before mu and ds
    float v = 0.f;
    if (ch < dof) v = (float)x[c * dof + ch] * sc.a[ch];
    else if (ch < 2 * dof) v = (float)t[c * dof + ch - dof] * sc.b[ch - dof];
    else if (pv && ch < 3 * dof) v = (float)pv[c * dof + ch - 2 * dof] * sp.a[ch - 2 * dof];
    else if (ch == nf * dof) v = mu;
    else if (ch == nf * dof + 1) v = ds;
    X0[e] = __float2bfloat16(v);
}

// Training target: the corrector's displacement from the secant predictor,
// (x1 - x0 - ds t) scaled per variable.
__global__ void target_kernel(int ncell, int dof, const double *__restrict__ x0, const double *__restrict__ t,
                              const double *__restrict__ x1, double ds, StateScales inv, float *__restrict__ tgt) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncell * dof) return;
    const int d = (int)(e % dof);
    tgt[e] = (float)((x1[e] - x0[e] - ds * t[e]) * inv.a[d]);
}

// Predictor: x0 + ds t + scale[d] * out[c][d].  Unknowns the branch does not
// move (secant tangent exactly zero: the pressure gauge, boundary-face
// velocities no equation changes) keep the secant value, so the corrector
// converges to the solution with the same gauge as the plain branch.
__global__ void unpack_kernel(int ncell, int dof, int np, const float *__restrict__ out,
                              const double *__restrict__ x0, const double *__restrict__ t, double ds, StateScales sc,
                              double *__restrict__ xp) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncell * dof) return;
    const long long c = e / dof;
    const int d = (int)(e % dof);
    const double tv = t[e];
    xp[e] = x0[e] + ds * tv + (tv != 0.0 ? sc.a[d] * (double)out[c * np + d] : 0.0);
}

// Adam on the FP32 master weights (update != 0), then the two BF16 layouts.
__global__ void adam_kernel(int kp, int np, float *__restrict__ w, float *__restrict__ bias,
                            const float *__restrict__ grad, float *__restrict__ m, float *__restrict__ v, float lr,
                            float b1, float b2, float eps, float c1, float c2, float gscale, int update,
                            __nv_bfloat16 *__restrict__ bf, __nv_bfloat16 *__restrict__ bb) {
    const int pairs = kp * np;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 28 * pairs) return;
    const int tap = e / pairs, p = e % pairs, ci = p / np, co = p % np;
    if (tap == 27 && ci != 0) return;
    float *wp = tap < 27 ? w + e : bias + co;
    float wv = *wp;
    if (update) {
        const float gr = grad[e] * gscale;
        const float mm = b1 * m[e] + (1.f - b1) * gr;
        const float vv = b2 * v[e] + (1.f - b2) * gr * gr;
        m[e] = mm;
        v[e] = vv;
        wv -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        *wp = wv;
    }
    if (tap < 27) {
        const __nv_bfloat16 h = __float2bfloat16(wv);
        bf[((size_t)tap * np + co) * kp + ci] = h;
        bb[((size_t)(26 - tap) * kp + ci) * np + co] = h;
    }
}

static inline int blocks(long long n, int b) { return (int)((n + b - 1) / b); }

static inline bool ch_ok(int c) { return c == 16 || c == 32; }

static inline bool grid_ok(int nx, int ny, int nz) {
    return nx > 0 && ny > 0 && nz > 0 && (long long)nx * ny * nz < (1LL << 26);
}

static inline int nchunks(int ncell) { return (ncell + WG_CELLS - 1) / WG_CELLS; }

template <int KP, int NP>
static int launch_conv(int ncell, int nx, int ny, int nz, const __nv_bfloat16 *x, const __nv_bfloat16 *w,
                       const float *bias, float *z, __nv_bfloat16 *a, int relu, cudaStream_t s) {
    const size_t sm = ConvShape<KP, NP>::smem;
    if (sm > 48 * 1024 &&
        cudaFuncSetAttribute((const void *)conv_kernel<KP, NP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm) != cudaSuccess) {
        cudaGetLastError();
        return TF_ERR_CUDA;
    }
    conv_kernel<KP, NP><<<blocks(ncell, CV_M), CV_THREADS, sm, s>>>(nx, ny, nz, x, w, bias, z, a, relu);
    launched();
    return TF_OK;
}

}  // namespace sg
}  // namespace tf

using namespace tf;
using namespace tf::sg;

extern "C" int tf_sg_conv(int nx, int ny, int nz, int kp, int np, const void *d_x, const void *d_w,
                          const float *d_bias, float *d_z, void *d_a, int relu, tf_stream_t stream) {
    if (!grid_ok(nx, ny, nz) || !ch_ok(kp) || !ch_ok(np) || !d_x || !d_w || (!d_z && !d_a)) return TF_ERR_ARG;
    const int ncell = nx * ny * nz;
    const auto *x = static_cast<const __nv_bfloat16 *>(d_x);
    const auto *w = static_cast<const __nv_bfloat16 *>(d_w);
    auto *a = static_cast<__nv_bfloat16 *>(d_a);
    cudaStream_t s = (cudaStream_t)stream;
    int e;
    if (kp == 16 && np == 16) e = launch_conv<16, 16>(ncell, nx, ny, nz, x, w, d_bias, d_z, a, relu, s);
    else if (kp == 16) e = launch_conv<16, 32>(ncell, nx, ny, nz, x, w, d_bias, d_z, a, relu, s);
    else if (np == 16) e = launch_conv<32, 16>(ncell, nx, ny, nz, x, w, d_bias, d_z, a, relu, s);
    else e = launch_conv<32, 32>(ncell, nx, ny, nz, x, w, d_bias, d_z, a, relu, s);
    return e ? e : cuda_status();
}

extern "C" size_t tf_sg_wgrad_workspace_bytes(int ncell, int kp, int np) {
    if (ncell <= 0 || kp <= 0 || np <= 0) return 0;
    return (size_t)nchunks(ncell) * 28 * kp * np * sizeof(float);
}

extern "C" int tf_sg_wgrad(int nx, int ny, int nz, int kp, int np, const void *d_x, const float *d_dz,
                           float *d_grad, int accumulate, void *d_work, size_t work_bytes, tf_stream_t stream) {
    if (!grid_ok(nx, ny, nz) || !ch_ok(kp) || !ch_ok(np) || !d_x || !d_dz || !d_grad || !d_work) return TF_ERR_ARG;
    const int ncell = nx * ny * nz;
    if (work_bytes < tf_sg_wgrad_workspace_bytes(ncell, kp, np)) return TF_ERR_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    float *part = static_cast<float *>(d_work);
    wgrad_kernel<<<dim3(nchunks(ncell), 28), WG_THREADS, 0, s>>>(nx, ny, nz, static_cast<const __nv_bfloat16 *>(d_x),
                                                                 kp, d_dz, np, part);
    const int m = 28 * kp * np;
    reduce_kernel<<<blocks(m, 256), 256, 0, s>>>(nchunks(ncell), m, part, d_grad, accumulate);
    launched(2);
    return cuda_status();
}

extern "C" size_t tf_sg_loss_workspace_bytes(int ncell, int np) {
    if (ncell <= 0 || np <= 0) return 0;
    return (size_t)blocks((long long)ncell * np, 256) * sizeof(double);
}

extern "C" int tf_sg_loss(int ncell, int dof, int np, const float *d_out, const float *d_tgt, float *d_dzf,
                          void *d_dzh, double *d_loss, void *d_work, size_t work_bytes, tf_stream_t stream) {
    if (ncell <= 0 || dof <= 0 || dof > np || !ch_ok(np) || !d_out || !d_tgt || !d_dzf || !d_dzh || !d_loss ||
        !d_work)
        return TF_ERR_ARG;
    if (work_bytes < tf_sg_loss_workspace_bytes(ncell, np)) return TF_ERR_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = blocks((long long)ncell * np, 256);
    const double count = (double)ncell * dof;
    auto *part = static_cast<double *>(d_work);
    loss_kernel<<<nb, 256, 0, s>>>(ncell, dof, np, d_out, d_tgt, (float)(2.0 / count), d_dzf,
                                   static_cast<__nv_bfloat16 *>(d_dzh), part);
    sum_kernel<<<1, 256, 0, s>>>(nb, part, 1.0 / count, d_loss);
    launched(2);
    return cuda_status();
}

extern "C" int tf_sg_act_grad(long long n, const float *d_da, const float *d_z, float *d_dzf, void *d_dzh,
                              tf_stream_t stream) {
    if (n <= 0 || !d_da || !d_z || !d_dzf || !d_dzh) return TF_ERR_ARG;
    act_grad_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(n, d_da, d_z, d_dzf,
                                                                        static_cast<__nv_bfloat16 *>(d_dzh));
    launched();
    return cuda_status();
}

extern "C" int tf_sg_pack(int ncell, int dof, int kp, const double *d_x, const double *d_t, const double *d_p,
                          const float *sx, const float *st, const float *sp, float mu, float ds, void *d_x0,
                          tf_stream_t stream) {
    const int nf = d_p ? 3 : 2;
    if (ncell <= 0 || dof <= 0 || dof > MAX_DOF || nf * dof + 2 > kp || !ch_ok(kp) || !d_x || !d_t || !sx || !st ||
        (d_p && !sp) || !d_x0)
        return TF_ERR_ARG;
    FieldScales sc = {}, spc = {};
    for (int d = 0; d < dof; ++d) {
        sc.a[d] = sx[d];
        sc.b[d] = st[d];
        spc.a[d] = d_p ? sp[d] : 0.f;
    }
    pack_kernel<<<blocks((long long)ncell * kp, 256), 256, 0, (cudaStream_t)stream>>>(
        ncell, dof, kp, d_x, d_t, d_p, sc, spc, mu, ds, static_cast<__nv_bfloat16 *>(d_x0));
    launched();
    return cuda_status();
}

extern "C" int tf_sg_target(int ncell, int dof, const double *d_x0, const double *d_t, const double *d_x1, double ds,
                            const double *inv_scale, float *d_tgt, tf_stream_t stream) {
    if (ncell <= 0 || dof <= 0 || dof > MAX_DOF || !d_x0 || !d_t || !d_x1 || !inv_scale || !d_tgt) return TF_ERR_ARG;
    StateScales inv = {};
    for (int d = 0; d < dof; ++d) inv.a[d] = inv_scale[d];
    target_kernel<<<blocks((long long)ncell * dof, 256), 256, 0, (cudaStream_t)stream>>>(ncell, dof, d_x0, d_t, d_x1,
                                                                                          ds, inv, d_tgt);
    launched();
    return cuda_status();
}

extern "C" int tf_sg_unpack(int ncell, int dof, int np, const float *d_out, const double *d_x0, const double *d_t,
                            double ds, const double *scale, double *d_xp, tf_stream_t stream) {
    if (ncell <= 0 || dof <= 0 || dof > MAX_DOF || dof > np || !ch_ok(np) || !d_out || !d_x0 || !d_t || !scale ||
        !d_xp)
        return TF_ERR_ARG;
    StateScales sc = {};
    for (int d = 0; d < dof; ++d) sc.a[d] = scale[d];
    unpack_kernel<<<blocks((long long)ncell * dof, 256), 256, 0, (cudaStream_t)stream>>>(ncell, dof, np, d_out, d_x0,
                                                                                          d_t, ds, sc, d_xp);
    launched();
    return cuda_status();
}

extern "C" int tf_sg_adam(int kp, int np, float *d_w, float *d_bias, const float *d_grad, float *d_m, float *d_v,
                          float lr, float beta1, float beta2, float eps, int step, float grad_scale, void *d_wf,
                          void *d_wb, tf_stream_t stream) {
    if (!ch_ok(kp) || !ch_ok(np) || !d_w || !d_bias || !d_wf || !d_wb || step < 0) return TF_ERR_ARG;
    if (step > 0 && (!d_grad || !d_m || !d_v)) return TF_ERR_ARG;
    float c1 = 1.f, c2 = 1.f;
    if (step > 0) {
        c1 = 1.f - powf(beta1, (float)step);
        c2 = 1.f - powf(beta2, (float)step);
    }
    const int n = 28 * kp * np;
    adam_kernel<<<blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(
        kp, np, d_w, d_bias, d_grad, d_m, d_v, lr, beta1, beta2, eps, c1, c2, grad_scale, step > 0 ? 1 : 0,
        static_cast<__nv_bfloat16 *>(d_wf), static_cast<__nv_bfloat16 *>(d_wb));
    launched();
    return cuda_status();
}
