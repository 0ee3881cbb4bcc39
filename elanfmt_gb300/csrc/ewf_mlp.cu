// ewf_mlp.cu -- kernels of the learned Green's-function surrogate (training and inference).
//
// A small MLP maps (source x, y, depth, receiver offset, azimuth) to the 6 x 3 x nt elementary
// Green's-function seismograms; the solver generates its training data and measures its error.
// Everything here works on caller-owned device buffers (plain pointers):
//   ewf_mlp_gemm        C[M,N] = A[M,K] . B[N,K]^T (+ bias), bf16 operands on the tcgen05 tensor
//                       cores (TMA-fed, fp32 accumulator in tensor memory), epilogue: fp32 out,
//                       bf16 out, pre-activation out, GELU
//   ewf_mlp_transpose   bf16 [R,C] -> [C,R] (so every product is an A.B^T GEMM)
//   ewf_mlp_gelu_grad   dX = dY * GELU'(pre)  (bf16 out)
//   ewf_mlp_bias_grad   db[n] = sum_m dY[m,n]
//   ewf_mlp_mse_grad    dY = 2 (Y - T) / count (bf16), and the loss sum
//   ewf_mlp_adam        Adam step on fp32 master weights, refreshing the bf16 copy
//   ewf_mlp_combine     out[m,o,t] = sum_f R[m,o,f] G[m,f,t]: per-sample mixing of the predicted
//                       fundamental traces into the 18 moment-tensor x component traces
// The GEMM requires M, N multiples of 128 and K a multiple of 32 (checked on the host).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>
#include <mutex>
#include <set>

#include "ewf_umma.h"
#include "ewfd.h"
#include "ewfd_internal.h"

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// ---------------------------------------------------------------------------------------------
// tcgen05 GEMM: C[M,N] = A[M,K] . B[N,K]^T on the 5th-generation tensor cores.  Persistent: one
// CTA per SM walks the 128 x BN tiles of C (BN = 256, or 128 when N is not a multiple of 256).
// Two fp32 accumulators of 128 lanes x BN columns in tensor memory, so the epilogue of one tile
// overlaps the MMAs of the next.  Warp roles, 192 threads:
//   warp 0, one lane: TMA producer -- per k-stage one 2-D bulk tensor copy per operand (128-byte
//     swizzle, ewf_umma.h) into the next free slot of a 4-stage ring, completing on that slot's
//     "full" mbarrier; the ring runs on across tiles;
//   warp 1, one lane: MMA issuer -- waits for a free accumulator ("acc_empty"), then per stage for
//     "full", issues 4 tcgen05.mma (K = 16 each) and commits them to the slot's "empty" mbarrier
//     (freeing it for the producer); after the tile's last stage commits "acc_full";
//   warps 2-5: epilogue -- wait for "acc_full", read the accumulator with tcgen05.ld (warp w owns
//     TMEM lanes 32 (w % 4) ..), add the bias, GELU, write the requested outputs, release the
//     accumulator ("acc_empty", one arrival per warp).  When only the fp32 C is wanted and every
//     SM has two tiles or more, each warp stages 32 rows x 64 columns in shared memory and writes
//     them with one TMA store (row-contiguous, asynchronous); otherwise every lane stores its row.
// K beyond the last full stage would be read as zeros (the tensor map's out-of-bounds fill); the
// host accepts K multiples of 32.  Every mbarrier wait is bounded (g_umma_wait_limit polls): on
// timeout the wait raises g_umma_err and gives up (the outputs of that launch are then invalid,
// ewf_mlp_status reports it), and no later wait of the launch waits at all.  Before the CTA frees
// its tensor memory and returns, the producer waits (again bounded, with a fixed limit) for the
// last TMA loads it issued and the MMA issuer for every MMA it issued, whether or not a wait
// gave up.  Test hook (ewf_mlp_test_hold): the MMA issuer of CTA 0 withholds the accumulator-
// ready signal of one of its tiles, so the epilogue's wait on it runs out.
// ---------------------------------------------------------------------------------------------
__device__ int g_umma_err = 0;
constexpr int kWaitPolls = 1 << 22;
__device__ int g_umma_wait_limit = kWaitPolls;
__device__ int g_umma_hold = -1;  // tile (CTA-local index) of CTA 0 whose acc_full is withheld; -1: none

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(b)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool umma_failed() { return *(volatile int *)&g_umma_err != 0; }
// Bounded wait; gives up at once when another wait of the launch has already given up.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity)
{
    const int limit = *(volatile int *)&g_umma_wait_limit;
    for (int i = 0; i < limit; ++i) {
        if (mbar_try_wait(b, parity)) return true;
        if ((i & 1023) == 1023 && umma_failed()) break;
    }
    atomicExch(&g_umma_err, 1);
    return false;
}
// Wait for asynchronous work this thread issued itself (fixed bound: the work always completes).
__device__ __forceinline__ void mbar_drain(uint64_t *b, uint32_t parity)
{
    for (int i = 0; i < kWaitPolls; ++i)
        if (mbar_try_wait(b, parity)) return;
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
                     smem_u32(dst)),
                 "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t accum)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
                 "l"(da), "l"(db), "r"(idesc), "r"(accum)
                 : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *b)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
}
// 16 consecutive fp32 accumulator columns of this thread's lane (load and wait in one block so
// no use of the values can be scheduled before the wait)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
                 "tcgen05.wait::ld.sync.aligned;"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                 : "r"(taddr)
                 : "memory");
}

template <int BN>
__global__ void __launch_bounds__(ewf_umma::THREADS, 1)
    k_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, const __grid_constant__ CUtensorMap mapC, int tma_c,
             const float *__restrict__ bias, float *__restrict__ Cf, __nv_bfloat16 *__restrict__ Cb, float *__restrict__ Pre,
             int M, int N, int K, int act)
{
    namespace U = ewf_umma;
    constexpr int STAGE = U::a_bytes() + BN * U::ROW_BYTES;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t full[U::STAGES], empty[U::STAGES], acc_full[2], acc_empty[2], mma_drain;
    __shared__ uint32_t s_tmem;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int tiles_n = N / BN, tiles = (M / U::BM) * tiles_n;
    const int nk = (K + U::BK - 1) / U::BK;

    if (tid == 0) {
        for (int s = 0; s < U::STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);  // one arrival per epilogue warp
        }
        mbar_init(&mma_drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)), "r"(2 * BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {  // TMA producer: every k-stage of every tile of this CTA, one ring
            int g = 0;
            for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
                const int m0 = (t / tiles_n) * U::BM, n0 = (t % tiles_n) * BN;
                for (int kt = 0; kt < nk; ++kt, ++g) {
                    const int s = U::ring_slot(g);
                    if (U::ring_needs_free(g) && !mbar_wait(&empty[s], U::ring_free_parity(g))) { ok = false; break; }
                    uint8_t *As = smem + s * STAGE;
                    mbar_expect_tx(&full[s], STAGE);
                    tma_load_2d(As, &mapA, kt * U::BK, m0, &full[s]);
                    tma_load_2d(As + U::a_bytes(), &mapB, kt * U::BK, n0, &full[s]);
                }
            }
            // the loads issued last into each slot land before the CTA's shared memory goes
            for (int q = (g > U::STAGES ? g - U::STAGES : 0); q < g; ++q)
                mbar_drain(&full[U::ring_slot(q)], U::ring_full_parity(q));
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            const uint32_t idesc = U::instr_desc_bf16_f32(U::BM, BN);
            const int hold = blockIdx.x == 0 ? *(volatile int *)&g_umma_hold : -1;
            int g = 0, i = 0;
            for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x, ++i) {
                const int b = U::acc_buf(i);
                if (U::acc_needs_free(i) && !mbar_wait(&acc_empty[b], U::acc_free_parity(i))) { ok = false; break; }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * BN);
                for (int kt = 0; kt < nk; ++kt, ++g) {
                    const int s = U::ring_slot(g);
                    if (!mbar_wait(&full[s], U::ring_full_parity(g))) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(smem + s * STAGE), b0 = a0 + U::a_bytes();
                    for (int j = 0; j < U::BK / U::MMA_K; ++j)
                        umma_bf16(d, U::smem_desc_sw128(a0 + 32 * j), U::smem_desc_sw128(b0 + 32 * j), idesc,
                                  (kt > 0 || j > 0) ? 1u : 0u);
                    umma_commit(&empty[s]);
                }
                if (!ok) break;
                if (i != hold) umma_commit(&acc_full[b]);
            }
            // every MMA issued completes before the tensor memory is freed
            umma_commit(&mma_drain);
            mbar_drain(&mma_drain, 0);
        }
    } else {  // epilogue warps 2..5: TMEM lane quarter q = warp % 4
        const int q = warp & 3;
        int i = 0;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++i) {
            const int b = U::acc_buf(i);
            const bool got = !umma_failed() && mbar_wait(&acc_full[b], U::acc_full_parity(i));
            tc_fence_after();
            const int m0 = (t / tiles_n) * U::BM, n0 = (t % tiles_n) * BN;
            const int row = m0 + 32 * q + lane;
            if (tma_c) {
                // stage 32 rows x 64 columns of this warp in shared memory, store them with one TMA box
                float *buf = reinterpret_cast<float *>(smem + U::STAGES * STAGE) + (warp - 2) * (32 * 64);
#pragma unroll 1
                for (int c0 = 0; c0 < BN; c0 += 64) {
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
#pragma unroll 1
                    for (int h = 0; h < 64; h += 16) {
                        uint32_t v[16];
                        tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN + c0 + h), v);
#pragma unroll
                        for (int e = 0; e < 16; e += 4) {
                            float x0 = got ? __uint_as_float(v[e]) : __int_as_float(0x7fc00000);
                            float x1 = got ? __uint_as_float(v[e + 1]) : __int_as_float(0x7fc00000);
                            float x2 = got ? __uint_as_float(v[e + 2]) : __int_as_float(0x7fc00000);
                            float x3 = got ? __uint_as_float(v[e + 3]) : __int_as_float(0x7fc00000);
                            if (bias) {
                                x0 += bias[n0 + c0 + h + e];
                                x1 += bias[n0 + c0 + h + e + 1];
                                x2 += bias[n0 + c0 + h + e + 2];
                                x3 += bias[n0 + c0 + h + e + 3];
                            }
                            if (act == 1) {
                                x0 = gelu(x0);
                                x1 = gelu(x1);
                                x2 = gelu(x2);
                                x3 = gelu(x3);
                            }
                            *reinterpret_cast<float4 *>(buf + lane * 64 + h + e) = make_float4(x0, x1, x2, x3);
                        }
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) {
                        asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                                         (uint64_t)&mapC),
                                     "r"(n0 + c0), "r"(m0 + 32 * q), "r"(smem_u32(buf))
                                     : "memory");
                        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    }
                }
            } else {
    #pragma unroll 1
                for (int c0 = 0; c0 < BN; c0 += 16) {
                    uint32_t v[16];
                    tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * BN + c0), v);
                    float x[16];
    #pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        x[e] = got ? __uint_as_float(v[e]) : __int_as_float(0x7fc00000);
                        if (bias) x[e] += bias[n0 + c0 + e];
                    }
                    const size_t o = (size_t)row * N + n0 + c0;
                    if (Pre)
    #pragma unroll
                        for (int e = 0; e < 16; e += 4) *reinterpret_cast<float4 *>(Pre + o + e) = make_float4(x[e], x[e + 1], x[e + 2], x[e + 3]);
                    if (act == 1)
    #pragma unroll
                        for (int e = 0; e < 16; ++e) x[e] = gelu(x[e]);
                    if (Cf)
    #pragma unroll
                        for (int e = 0; e < 16; e += 4) *reinterpret_cast<float4 *>(Cf + o + e) = make_float4(x[e], x[e + 1], x[e + 2], x[e + 3]);
                    if (Cb)
    #pragma unroll
                        for (int e = 0; e < 16; e += 2) *reinterpret_cast<__nv_bfloat162 *>(Cb + o + e) = __floats2bfloat162_rn(x[e], x[e + 1]);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acc_empty[b])) : "memory");
        }
    }
    if (tma_c && warp >= 2 && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
    }
}
int check(cudaError_t e, const char *what);

// 2-D tensor map of a K-major bf16 operand [rows, K] with boxes of BK x box_rows and the 128-byte swizzle
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn tensor_map_encoder()
{
    static EncodeTiledFn enc = nullptr;
    if (!enc) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            fn && q == cudaDriverEntryPointSuccess)
            enc = (EncodeTiledFn)fn;
    }
    return enc;
}

int operand_map(CUtensorMap *m, const void *ptr, int rows, int K, int box_rows)
{
    const EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return ewf_fail(EWF_ERR_CUDA, "gemm: cuTensorMapEncodeTiled unavailable");
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)ewf_umma::BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? EWF_OK : ewf_fail(EWF_ERR_ARG, "gemm: tensor map rejected (CUresult %d)", (int)r);
}

// tensor map of the fp32 output [M, N] for the staged epilogue: boxes of 64 columns x 32 rows
int output_map(CUtensorMap *m, float *C, int M, int N)
{
    const EncodeTiledFn enc = tensor_map_encoder();
    if (!enc) return ewf_fail(EWF_ERR_CUDA, "gemm: cuTensorMapEncodeTiled unavailable");
    const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)M};
    const cuuint64_t strides[1] = {(cuuint64_t)N * 4};
    const cuuint32_t box[2] = {64, 32};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? EWF_OK : ewf_fail(EWF_ERR_ARG, "gemm: output tensor map rejected (CUresult %d)", (int)r);
}

constexpr int EPI_STAGE_BYTES = 4 * 32 * 64 * 4;  // four epilogue warps x 32 rows x 64 fp32

// The kernel's shared-memory attribute is a per-device setting: set once per device ordinal.
template <int BN>
int gemm_smem_attribute(int dev, int smem_max)
{
    static std::mutex mu;
    static std::set<int> done;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(dev)) return EWF_OK;
    const cudaError_t e = cudaFuncSetAttribute(k_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
    if (e != cudaSuccess) return check(e, "gemm smem attribute");
    done.insert(dev);
    return EWF_OK;
}

template <int BN>
int launch_gemm(const void *A, const void *B, const float *bias, float *Cf, void *Cb, float *pre, int M, int N, int K,
                int act, cudaStream_t stream)
{
    int dev = 0, sms = 0;
    int st = check(cudaGetDevice(&dev), "gemm device");
    if (st) return st;
    if ((st = gemm_smem_attribute<BN>(dev, ewf_umma::smem_bytes(BN) + EPI_STAGE_BYTES))) return st;
    alignas(64) CUtensorMap ma, mb, mc;
    if ((st = operand_map(&ma, A, M, K, ewf_umma::BM))) return st;
    if ((st = operand_map(&mb, B, N, K, BN))) return st;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (M / ewf_umma::BM) * (N / BN);
    const int grid = tiles < sms ? tiles : (sms > 0 ? sms : 1);  // one CTA per SM (shared memory bound)
    // staged TMA stores for an fp32-only output when every SM has two tiles or more (fewer: per-lane
    // stores win -- 12800 x 512 x 256, 1.3 tiles per SM: 199 against 161 TFLOP/s)
    const int tma_c = (Cf && !Cb && !pre && tiles >= 2 * sms) ? 1 : 0;
    memset(&mc, 0, sizeof(mc));
    if (tma_c && (st = output_map(&mc, Cf, M, N))) return st;
    const int smem = ewf_umma::smem_bytes(BN) + (tma_c ? EPI_STAGE_BYTES : 0);
    k_gemm<BN><<<grid, ewf_umma::THREADS, smem, stream>>>(ma, mb, mc, tma_c, bias, Cf, (__nv_bfloat16 *)Cb, pre, M, N, K,
                                                          act);
    return check(cudaGetLastError(), "gemm launch");
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
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 32)
        return ewf_fail(EWF_ERR_ARG, "gemm: M, N must be multiples of 128 and K of 32 (got %d %d %d)", M, N, K);
    if (act != 0 && act != 1) return ewf_fail(EWF_ERR_ARG, "gemm: act must be 0 or 1");
    if (((uintptr_t)A | (uintptr_t)B) & 15) return ewf_fail(EWF_ERR_ARG, "gemm: A and B must be 16-byte aligned");
    if (((uintptr_t)Cf | (uintptr_t)pre) & 15 || (uintptr_t)Cb & 3) return ewf_fail(EWF_ERR_ARG, "gemm: outputs misaligned");
    if (N % 256 == 0) return launch_gemm<256>(A, B, bias, Cf, Cb, pre, M, N, K, act, (cudaStream_t)stream);
    return launch_gemm<128>(A, B, bias, Cf, Cb, pre, M, N, K, act, (cudaStream_t)stream);
}

extern "C" int ewf_mlp_status(void)
{
    int e = 0;
    cudaError_t ce = cudaMemcpyFromSymbol(&e, g_umma_err, sizeof(int));
    if (ce != cudaSuccess) return check(ce, "gemm status");
    if (e) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_umma_err, &zero, sizeof(int));
        return ewf_fail(EWF_ERR_CUDA, "gemm: an mbarrier wait gave up (outputs of that launch are invalid)");
    }
    return EWF_OK;
}

extern "C" int ewf_mlp_test_hold(int32_t tile, int32_t polls)
{
    const int h = tile >= 0 ? tile : -1;
    const int v = (tile >= 0 && polls > 0) ? polls : kWaitPolls;
    int st = check(cudaMemcpyToSymbol(g_umma_wait_limit, &v, sizeof(int)), "gemm wait limit");
    if (!st) st = check(cudaMemcpyToSymbol(g_umma_hold, &h, sizeof(int)), "gemm hold");
    return st;
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
