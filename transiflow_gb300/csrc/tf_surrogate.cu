// Learned continuation predictor: a stack of 3x3x3 convolutions over the
// cell grid that proposes the correction to the secant predictor of
// pseudo-arclength continuation.  Activations are channels-last
// ([cell][channel], cell = i + nx*(j + ny*k), the ordering of the state
// vector), operands are BF16 and every product is accumulated in FP32 on the
// tensor cores (mma.sync m16n8k16).  Training runs here too: the gradient
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

namespace tf {
namespace sg {

constexpr int CONV_WARPS = 4;     // 16 cells per warp, 64 per CTA
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

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *p) {
    return __ldg(reinterpret_cast<const unsigned int *>(p));
}

// D = A * B + D, A 16x16 (row), B 16x8 (col), BF16 operands, FP32 accumulators.
__device__ __forceinline__ void mma_bf16(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Neighbour of cell (i, j, k) across tap, or -1 outside the grid (zero padding).
__device__ __forceinline__ int neighbour(int i, int j, int k, int tap, int nx, int ny, int nz) {
    const int a = i + tap % 3 - 1, b = j + (tap / 3) % 3 - 1, c = k + tap / 9 - 1;
    if (a < 0 || a >= nx || b < 0 || b >= ny || c < 0 || c >= nz) return -1;
    return a + nx * (b + ny * c);
}

// One 3x3x3 convolution as an implicit GEMM: rows are cells, K runs over
// (tap, input channel), N over output channels.  A warp owns 16 consecutive
// cells and all NP output channels.  Lane (g = lane/4, t = lane%4) holds the
// A fragment of cells base+g and base+g+8 at input channels 2t, 2t+1, 2t+8,
// 2t+9 of each 16-channel chunk, and the B fragment of output channel g at
// the same input channels.  Z (FP32, optional) receives conv + bias, A (BF16,
// optional) relu(conv + bias) when relu is set, else conv + bias.
template <int KC, int NT>
__global__ void __launch_bounds__(32 * CONV_WARPS)
conv_kernel(int nx, int ny, int nz, const __nv_bfloat16 *__restrict__ X, const __nv_bfloat16 *__restrict__ B,
            const float *__restrict__ bias, float *__restrict__ Z, __nv_bfloat16 *__restrict__ A, int relu) {
    constexpr int KP = 16 * KC, NP = 8 * NT;
    const int ncell = nx * ny * nz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int base = (blockIdx.x * CONV_WARPS + warp) * 16;
    if (base >= ncell) return;  // the whole warp leaves: mma.sync needs all 32 lanes
    const int r0 = base + g, r1 = base + g + 8;
    const bool v0 = r0 < ncell, v1 = r1 < ncell;
    const int nxy = nx * ny;
    const int i0 = r0 % nx, j0 = (r0 / nx) % ny, k0 = r0 / nxy;
    const int i1 = r1 % nx, j1 = (r1 / nx) % ny, k1 = r1 / nxy;
    float acc[NT][4];
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
    for (int tap = 0; tap < 27; ++tap) {
        const int n0 = v0 ? neighbour(i0, j0, k0, tap, nx, ny, nz) : -1;
        const int n1 = v1 ? neighbour(i1, j1, k1, tap, nx, ny, nz) : -1;
        const __nv_bfloat16 *x0 = X + (size_t)(n0 < 0 ? 0 : n0) * KP + 2 * t;
        const __nv_bfloat16 *x1 = X + (size_t)(n1 < 0 ? 0 : n1) * KP + 2 * t;
        const __nv_bfloat16 *bt = B + ((size_t)tap * NP + g) * KP + 2 * t;
#pragma unroll
        for (int kc = 0; kc < KC; ++kc) {
            const uint32_t a0 = n0 >= 0 ? ld_pair(x0 + 16 * kc) : 0u;
            const uint32_t a1 = n1 >= 0 ? ld_pair(x1 + 16 * kc) : 0u;
            const uint32_t a2 = n0 >= 0 ? ld_pair(x0 + 16 * kc + 8) : 0u;
            const uint32_t a3 = n1 >= 0 ? ld_pair(x1 + 16 * kc + 8) : 0u;
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
                const __nv_bfloat16 *bp = bt + (size_t)nt * 8 * KP + 16 * kc;
                mma_bf16(acc[nt], a0, a1, a2, a3, ld_pair(bp), ld_pair(bp + 8));
            }
        }
    }
#pragma unroll
    for (int nt = 0; nt < NT; ++nt) {
        const int col = nt * 8 + 2 * t;
        const float b0 = bias ? bias[col] : 0.f, b1 = bias ? bias[col + 1] : 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = h ? r1 : r0;
            if (!(h ? v1 : v0)) continue;
            const float z0 = acc[nt][2 * h] + b0, z1 = acc[nt][2 * h + 1] + b1;
            if (Z) *reinterpret_cast<float2 *>(Z + (size_t)r * NP + col) = make_float2(z0, z1);
            if (A) {
                const float y0 = relu ? fmaxf(z0, 0.f) : z0, y1 = relu ? fmaxf(z1, 0.f) : z1;
                *reinterpret_cast<__nv_bfloat162 *>(A + (size_t)r * NP + col) = __floats2bfloat162_rn(y0, y1);
            }
        }
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
                            FieldScales sc, float mu, float ds, __nv_bfloat16 *__restrict__ X0) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)ncell * kp) return;
    const long long c = e / kp;
    const int ch = (int)(e % kp);
    float v = 0.f;
    if (ch < dof) v = (float)x[c * dof + ch] * sc.a[ch];
    else if (ch < 2 * dof) v = (float)t[c * dof + ch - dof] * sc.b[ch - dof];
    else if (ch == 2 * dof) v = mu;
    else if (ch == 2 * dof + 1) v = ds;
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

}  // namespace sg
}  // namespace tf

using namespace tf;
using namespace tf::sg;

extern "C" int tf_sg_conv(int nx, int ny, int nz, int kp, int np, const void *d_x, const void *d_w,
                          const float *d_bias, float *d_z, void *d_a, int relu, tf_stream_t stream) {
    if (!grid_ok(nx, ny, nz) || !ch_ok(kp) || !ch_ok(np) || !d_x || !d_w || (!d_z && !d_a)) return TF_ERR_ARG;
    const int ncell = nx * ny * nz;
    const int grid = blocks(ncell, 16 * CONV_WARPS);
    const auto *x = static_cast<const __nv_bfloat16 *>(d_x);
    const auto *w = static_cast<const __nv_bfloat16 *>(d_w);
    auto *a = static_cast<__nv_bfloat16 *>(d_a);
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = 32 * CONV_WARPS;
    if (kp == 16 && np == 16) conv_kernel<1, 2><<<grid, threads, 0, s>>>(nx, ny, nz, x, w, d_bias, d_z, a, relu);
    else if (kp == 16) conv_kernel<1, 4><<<grid, threads, 0, s>>>(nx, ny, nz, x, w, d_bias, d_z, a, relu);
    else if (np == 16) conv_kernel<2, 2><<<grid, threads, 0, s>>>(nx, ny, nz, x, w, d_bias, d_z, a, relu);
    else conv_kernel<2, 4><<<grid, threads, 0, s>>>(nx, ny, nz, x, w, d_bias, d_z, a, relu);
    launched();
    return cuda_status();
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

extern "C" int tf_sg_pack(int ncell, int dof, int kp, const double *d_x, const double *d_t, const float *sx,
                          const float *st, float mu, float ds, void *d_x0, tf_stream_t stream) {
    if (ncell <= 0 || dof <= 0 || dof > MAX_DOF || 2 * dof + 2 > kp || !ch_ok(kp) || !d_x || !d_t || !sx || !st ||
        !d_x0)
        return TF_ERR_ARG;
    FieldScales sc = {};
    for (int d = 0; d < dof; ++d) {
        sc.a[d] = sx[d];
        sc.b[d] = st[d];
    }
    pack_kernel<<<blocks((long long)ncell * kp, 256), 256, 0, (cudaStream_t)stream>>>(
        ncell, dof, kp, d_x, d_t, sc, mu, ds, static_cast<__nv_bfloat16 *>(d_x0));
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
