// ewf_mlp.cu -- kernels of the learned Green's-function surrogate (training and inference).
//
// A small MLP maps (source x, y, depth, receiver offset, azimuth) to the 6 x 3 x nt elementary
// Green's-function seismograms; the solver generates its training data and measures its error.
// Everything here works on caller-owned device buffers (plain pointers):
//   ewf_mlp_gemm        C[M,N] = A[M,K] . B[N,K]^T (+ bias), bf16 operands on the tensor cores
//                       (mma.sync m16n8k16, fp32 accumulation), epilogue: fp32 out, bf16 out,
//                       pre-activation out, GELU
//   ewf_mlp_transpose   bf16 [R,C] -> [C,R] (so every product is an A.B^T GEMM)
//   ewf_mlp_gelu_grad   dX = dY * GELU'(pre)  (bf16 out)
//   ewf_mlp_bias_grad   db[n] = sum_m dY[m,n]
//   ewf_mlp_mse_grad    dY = 2 (Y - T) / count (bf16), and the loss sum
//   ewf_mlp_adam        Adam step on fp32 master weights, refreshing the bf16 copy
//   ewf_mlp_combine     out[m,o,t] = sum_f R[m,o,f] G[m,f,t]: per-sample mixing of the predicted
//                       fundamental traces into the 18 moment-tensor x component traces
// Tile sizes require M, N multiples of 128 and K a multiple of 32 (checked).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ewfd.h"
#include "ewfd_internal.h"

namespace {

constexpr int BM = 128, BN = 128, BK = 32, PAD = 8;
constexpr int LDS = BK + PAD;  // bf16 elements per smem row

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3, const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float *d, const uint32_t *a, const uint32_t *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// 256 threads = 8 warps as 2 (M) x 4 (N); warp tile 64 x 32 = 4 x 4 mma tiles of 16 x 8.
__global__ void __launch_bounds__(256) k_gemm_nt(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B,
                                                  const float *__restrict__ bias, float *__restrict__ Cf,
                                                  __nv_bfloat16 *__restrict__ Cb, float *__restrict__ Pre, int M, int N,
                                                  int K, int act)
{
    __shared__ __align__(16) __nv_bfloat16 As[2][BM][LDS];
    __shared__ __align__(16) __nv_bfloat16 Bs[2][BN][LDS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 2, wn = warp & 3;  // warp position
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    float acc[4][4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;

    // each thread copies 2 x 16 B of A and of B per stage: row = chunk / 4, col = (chunk % 4) * 8
    auto load_stage = [&](int st, int k0) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int ch = tid + q * 256;
            const int r = ch >> 2, cc = (ch & 3) * 8;
            cp_async16(&As[st][r][cc], A + (size_t)(m0 + r) * K + k0 + cc);
            cp_async16(&Bs[st][r][cc], B + (size_t)(n0 + r) * K + k0 + cc);
        }
        cp_async_commit();
    };

    const int nk = K / BK;
    load_stage(0, 0);
    for (int kt = 0; kt < nk; ++kt) {
        const int st = kt & 1;
        cp_async_wait_all();
        __syncthreads();
        if (kt + 1 < nk) load_stage(st ^ 1, (kt + 1) * BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[4][4], bfr[4][2];
#pragma unroll
            for (int mi = 0; mi < 4; ++mi) {
                const int row = wm * 64 + mi * 16 + (lane & 15);
                const int col = kk + (lane >> 4) * 8;
                ldmatrix_x4(af[mi][0], af[mi][1], af[mi][2], af[mi][3], &As[st][row][col]);
            }
#pragma unroll
            for (int nj = 0; nj < 4; nj += 2) {
                // two n8 tiles: matrices (n 0-7, k 0-7), (n 0-7, k 8-15), (n 8-15, k 0-7), (n 8-15, k 8-15)
                const int row = wn * 32 + nj * 8 + (lane & 7) + ((lane >> 4) << 3);
                const int col = kk + ((lane >> 3) & 1) * 8;
                uint32_t r0, r1, r2, r3;
                ldmatrix_x4(r0, r1, r2, r3, &Bs[st][row][col]);
                bfr[nj][0] = r0;
                bfr[nj][1] = r1;
                bfr[nj + 1][0] = r2;
                bfr[nj + 1][1] = r3;
            }
#pragma unroll
            for (int mi = 0; mi < 4; ++mi)
#pragma unroll
                for (int nj = 0; nj < 4; ++nj) mma_bf16(acc[mi][nj], af[mi], bfr[nj]);
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int mi = 0; mi < 4; ++mi)
#pragma unroll
        for (int nj = 0; nj < 4; ++nj)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int row = m0 + wm * 64 + mi * 16 + (lane >> 2) + h * 8;
                const int col = n0 + wn * 32 + nj * 8 + (lane & 3) * 2;
                float v0 = acc[mi][nj][2 * h], v1 = acc[mi][nj][2 * h + 1];
                if (bias) {
                    v0 += bias[col];
                    v1 += bias[col + 1];
                }
                const size_t o = (size_t)row * N + col;
                if (Pre) {
                    Pre[o] = v0;
                    Pre[o + 1] = v1;
                }
                if (act == 1) {
                    v0 = gelu(v0);
                    v1 = gelu(v1);
                }
                if (Cf) {
                    Cf[o] = v0;
                    Cf[o + 1] = v1;
                }
                if (Cb) *reinterpret_cast<__nv_bfloat162 *>(Cb + o) = __floats2bfloat162_rn(v0, v1);
            }
}

__global__ void k_transpose(const __nv_bfloat16 *__restrict__ in, __nv_bfloat16 *__restrict__ out, int R, int Cc)
{
    __shared__ __nv_bfloat16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int r = r0 + y, c = c0 + threadIdx.x;
        if (r < R && c < Cc) t[y][threadIdx.x] = in[(size_t)r * Cc + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int c = c0 + y, r = r0 + threadIdx.x;
        if (r < R && c < Cc) out[(size_t)c * R + r] = t[threadIdx.x][y];
    }
}

__global__ void k_gelu_grad(const __nv_bfloat16 *__restrict__ dy, const float *__restrict__ pre, __nv_bfloat16 *__restrict__ dx,
                            size_t n)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        dx[e] = __float2bfloat16_rn(__bfloat162float(dy[e]) * gelu_grad(pre[e]));
}

__global__ void k_bias_grad(const __nv_bfloat16 *__restrict__ dy, float *__restrict__ db, int M, int N)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; ++m) s += __bfloat162float(dy[(size_t)m * N + n]);
    db[n] = s;
}

// dY = 2 (Y - T) / count; loss partial sums (one per block) into part[blockIdx.x]
__global__ void k_mse_grad(const float *__restrict__ y, const float *__restrict__ t, __nv_bfloat16 *__restrict__ dy, size_t n,
                           float scale, float *__restrict__ part)
{
    __shared__ float red[256];
    float s = 0.f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float d = y[e] - t[e];
        s += d * d;
        dy[e] = __float2bfloat16_rn(2.f * d * scale);
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v, const float *__restrict__ g,
                       __nv_bfloat16 *__restrict__ wb, size_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float wd)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float ge = g[e] + wd * w[e];
        const float me = b1 * m[e] + (1.f - b1) * ge;
        const float ve = b2 * v[e] + (1.f - b2) * ge * ge;
        m[e] = me;
        v[e] = ve;
        const float we = w[e] - lr * (me / c1) / (sqrtf(ve / c2) + eps);
        w[e] = we;
        if (wb) wb[e] = __float2bfloat16_rn(we);
    }
}

unsigned blocks_for(size_t n) { return (unsigned)((n + 255) / 256 < 152 * 32 ? (n + 255) / 256 : 152 * 32); }

// One CTA per (sample, 256-sample slice of the time axis); the sample's mixing matrix sits in
// shared memory, every thread mixes one time sample (loads and stores coalesced along t).
constexpr int COMBINE_MAX = 2048;
__global__ void k_combine(const float *__restrict__ R, const float *__restrict__ G, float *__restrict__ out, int nout, int nin,
                          int T)
{
    __shared__ float r[COMBINE_MAX];
    const long long m = blockIdx.y;
    for (int e = threadIdx.x; e < nout * nin; e += blockDim.x) r[e] = R[m * nout * nin + e];
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const float *g = G + m * nin * T + t;
    float *o = out + m * nout * T + t;
    for (int a = 0; a < nout; ++a) {
        float acc = 0.f;
        for (int f = 0; f < nin; ++f) acc += r[a * nin + f] * g[(long long)f * T];
        o[(long long)a * T] = acc;
    }
}

int check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) return ewf_fail(EWF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return EWF_OK;
}

}  // namespace

extern "C" int ewf_mlp_gemm(const void *A, const void *B, const float *bias, float *Cf, void *Cb, float *pre, int32_t M,
                            int32_t N, int32_t K, int32_t act, void *stream)
{
    if (!A || !B || (!Cf && !Cb && !pre)) return ewf_fail(EWF_ERR_ARG, "gemm: NULL operand");
    if (M <= 0 || N <= 0 || K <= 0 || M % BM || N % BN || K % BK)
        return ewf_fail(EWF_ERR_ARG, "gemm: M, N must be multiples of %d and K of %d (got %d %d %d)", BM, BK, M, N, K);
    if (act != 0 && act != 1) return ewf_fail(EWF_ERR_ARG, "gemm: act must be 0 or 1");
    k_gemm_nt<<<dim3(N / BN, M / BM), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, bias, Cf, (__nv_bfloat16 *)Cb, pre, M, N, K, act);
    return check(cudaGetLastError(), "gemm launch");
}

extern "C" int ewf_mlp_transpose(const void *in, void *out, int32_t rows, int32_t cols, void *stream)
{
    if (!in || !out || rows <= 0 || cols <= 0) return ewf_fail(EWF_ERR_ARG, "transpose: bad argument");
    k_transpose<<<dim3((cols + 31) / 32, (rows + 31) / 32), dim3(32, 8), 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)in, (__nv_bfloat16 *)out, rows, cols);
    return check(cudaGetLastError(), "transpose launch");
}

extern "C" int ewf_mlp_gelu_grad(const void *dy, const float *pre, void *dx, size_t n, void *stream)
{
    if (!dy || !pre || !dx) return ewf_fail(EWF_ERR_ARG, "gelu_grad: NULL");
    k_gelu_grad<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dy, pre, (__nv_bfloat16 *)dx, n);
    return check(cudaGetLastError(), "gelu_grad launch");
}

extern "C" int ewf_mlp_bias_grad(const void *dy, float *db, int32_t M, int32_t N, void *stream)
{
    if (!dy || !db || M <= 0 || N <= 0) return ewf_fail(EWF_ERR_ARG, "bias_grad: bad argument");
    k_bias_grad<<<(N + 255) / 256, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)dy, db, M, N);
    return check(cudaGetLastError(), "bias_grad launch");
}

// part must hold `nblocks` floats: one partial sum of squared differences per block
extern "C" int ewf_mlp_mse_grad(const float *y, const float *t, void *dy, size_t n, float scale, float *part, int32_t nblocks,
                                void *stream)
{
    if (!y || !t || !dy || !part || nblocks < 1) return ewf_fail(EWF_ERR_ARG, "mse_grad: bad argument");
    k_mse_grad<<<nblocks, 256, 0, (cudaStream_t)stream>>>(y, t, (__nv_bfloat16 *)dy, n, scale, part);
    return check(cudaGetLastError(), "mse_grad launch");
}

extern "C" int ewf_mlp_adam(float *w, float *m, float *v, const float *g, void *wb, size_t n, float lr, float b1, float b2,
                            float eps, int32_t step, float weight_decay, void *stream)
{
    if (!w || !m || !v || !g || step < 1) return ewf_fail(EWF_ERR_ARG, "adam: bad argument");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, (__nv_bfloat16 *)wb, n, lr, b1, b2, eps, c1, c2,
                                                            weight_decay);
    return check(cudaGetLastError(), "adam launch");
}

extern "C" int ewf_mlp_combine(const float *R, const float *G, float *out, int32_t M, int32_t nout, int32_t nin, int32_t T,
                               void *stream)
{
    if (!R || !G || !out || M <= 0 || nout <= 0 || nin <= 0 || T <= 0) return ewf_fail(EWF_ERR_ARG, "combine: bad argument");
    if (M > 65535) return ewf_fail(EWF_ERR_ARG, "combine: at most 65535 samples per call (got %d)", M);
    if ((long long)nout * nin > COMBINE_MAX)
        return ewf_fail(EWF_ERR_ARG, "combine: nout * nin must be <= %d (got %d x %d)", COMBINE_MAX, nout, nin);
    k_combine<<<dim3((T + 255) / 256, M), 256, 0, (cudaStream_t)stream>>>(R, G, out, nout, nin, T);
    return check(cudaGetLastError(), "combine launch");
}
