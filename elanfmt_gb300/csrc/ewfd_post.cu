// ewfd_post.cu -- seismogram post-processing: a cascade of second-order IIR sections (the
// Butterworth band-pass the isotropic MATLAB driver applies before comparing traces,
// vizme_FastBiotED_GPU3D_OK_2024_final.m:551-558, 579-582, 604-607, "sosfilt(sos, x)").
//
// Each section is the direct form II transposed recursion
//     y = b0 x + s1;   s1 = b1 x - a1 y + s2;   s2 = b2 x - a2 y
// with zero initial state, the sections applied one after the other (section 0 first).  The
// host and device versions perform the same operations in the same order (the library is built
// without FMA contraction), so they give the same bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include "ewfd.h"
#include "ewfd_internal.h"

namespace {

constexpr int MAXSEC = EWF_SOS_MAX_SECTIONS;

struct Sos {
    double c[MAXSEC][5];  // b0 b1 b2 a1 a2, normalised by a0
    int n;
};

int make_sos(const double *sos, int32_t nsec, Sos *out)
{
    if (!sos || nsec < 1 || nsec > MAXSEC) return ewf_fail(EWF_ERR_ARG, "sosfilt: 1..%d sections (got %d)", MAXSEC, nsec);
    out->n = nsec;
    for (int s = 0; s < nsec; ++s) {
        const double *r = sos + 6 * s;
        const double a0 = r[3];
        if (!(a0 != 0.0)) return ewf_fail(EWF_ERR_ARG, "sosfilt: section %d has a0 = 0", s);
        out->c[s][0] = r[0] / a0;
        out->c[s][1] = r[1] / a0;
        out->c[s][2] = r[2] / a0;
        out->c[s][3] = r[4] / a0;
        out->c[s][4] = r[5] / a0;
    }
    return EWF_OK;
}

// one trace in place; __host__ __device__ so that both paths run the same code
__host__ __device__ inline void filter_trace(const Sos &q, double *x, int64_t n)
{
    double s1[MAXSEC], s2[MAXSEC];
    for (int s = 0; s < q.n; ++s) s1[s] = s2[s] = 0.0;
    for (int64_t t = 0; t < n; ++t) {
        double v = x[t];
        for (int s = 0; s < q.n; ++s) {
            const double *c = q.c[s];
            const double y = c[0] * v + s1[s];
            s1[s] = c[1] * v - c[3] * y + s2[s];
            s2[s] = c[2] * v - c[4] * y;
            v = y;
        }
        x[t] = v;
    }
}

__global__ void k_sosfilt(const Sos q, double *__restrict__ x, int64_t ntr, int64_t n)
{
    const int64_t tr = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tr < ntr) filter_trace(q, x + tr * n, n);
}

}  // namespace

extern "C" int ewf_sosfilt(const double *sos, int32_t nsec, double *x, int64_t ntr, int64_t n)
{
    Sos q;
    int st = make_sos(sos, nsec, &q);
    if (st) return st;
    if ((!x && ntr * n > 0) || ntr < 0 || n < 0) return ewf_fail(EWF_ERR_ARG, "sosfilt: bad trace array");
    for (int64_t tr = 0; tr < ntr; ++tr) filter_trace(q, x + tr * n, n);
    return EWF_OK;
}

extern "C" int ewf_sosfilt_device(const double *sos, int32_t nsec, double *x, int64_t ntr, int64_t n, void *stream)
{
    Sos q;
    int st = make_sos(sos, nsec, &q);
    if (st) return st;
    if ((!x && ntr * n > 0) || ntr < 0 || n < 0) return ewf_fail(EWF_ERR_ARG, "sosfilt: bad trace array");
    if (ntr == 0 || n == 0) return EWF_OK;
    const unsigned blocks = (unsigned)((ntr + 63) / 64);
    k_sosfilt<<<blocks, 64, 0, (cudaStream_t)stream>>>(q, x, ntr, n);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ewf_fail(EWF_ERR_CUDA, "sosfilt launch: %s", cudaGetErrorString(e));
    return EWF_OK;
}
