// ewfd_staged.cu -- instances, tensor maps and launches of the staged form of the one-pass step
// (ewfd_staged.cuh).
#include "ewfd_staged.cuh"

#include <mutex>
#include <set>

namespace ewf {

typedef CUresult (*StagedEncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static StagedEncodeFn staged_encoder()
{
    static std::once_flag once;
    static StagedEncodeFn enc = nullptr;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            fn && q == cudaDriverEntryPointSuccess)
            enc = (StagedEncodeFn)fn;
    });
    return enc;
}

// 3-D map of one padded float field (sx x (ny + 3) x (nz + 3), allocation start = element
// (-hx, -1, -1)) with boxes of bx x by x 1; elements outside the field read as zero.
static bool field_map(CUtensorMap *m, void *alloc, int sx, int ny, int nz, int bx, int by)
{
    const StagedEncodeFn enc = staged_encoder();
    if (!enc || !alloc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)sx, (cuuint64_t)ny + 3, (cuuint64_t)nz + 3};
    const cuuint64_t strides[2] = {(cuuint64_t)sx * 4, (cuuint64_t)sx * 4 * ((cuuint64_t)ny + 3)};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, alloc, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool staged_encode(StagedPlan &plan, void *const f_alloc[9], void *const g_alloc[9], void *const m_alloc[12],
                   void *w3_alloc, int nmat_big, const int *mat_slots, bool w3, bool buoyancy, int sx, int ny, int nz)
{
    plan.ok = false;
    for (int par = 0; par < 2; ++par)
        for (int q = 0; q < 9; ++q)
            if (!field_map(&plan.maps[par].st[q], par ? g_alloc[q] : f_alloc[q], sx, ny, nz, SBW, SBH)) return false;
    for (int par = 0; par < 2; ++par) {
        for (int f = 0; f < nmat_big; ++f)
            if (!field_map(&plan.maps[par].mt[f], m_alloc[mat_slots[f]], sx, ny, nz, SBW, SBH)) return false;
        if (w3 && !field_map(&plan.maps[par].mt[nmat_big], w3_alloc, sx, ny, nz, SBW, SBH)) return false;
        if (buoyancy)
            for (int f = 0; f < 3; ++f)
                if (!field_map(&plan.maps[par].bu[f], m_alloc[9 + f], sx, ny, nz, SX, SY)) return false;
    }
    plan.ok = true;
    return true;
}

template <int MODEL, int DAMP>
bool staged_ready()
{
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count(dev)) return true;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        (size_t)optin < staged_smem_bytes<MODEL, DAMP>())
        return false;
    if (cudaFuncSetAttribute(k_staged<MODEL, DAMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)staged_smem_bytes<MODEL, DAMP>()) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    done.insert(dev);
    return true;
}

template <int MODEL, int DAMP>
cudaError_t staged_launch(const FusedArgs<float> &fa, const StagedPlan &plan, int parity, int hx, cudaStream_t stream)
{
    StagedParams sp;
    sp.fa = fa;
    sp.maps = plan.maps[parity];
    sp.hx = hx;
    const dim3 grd((fa.a.nx + SX - 1) / SX, (fa.a.ny + SY - 1) / SY, (fa.a.nz + fa.a.kchunk - 1) / fa.a.kchunk);
    k_staged<MODEL, DAMP><<<grd, dim3(SX, SY), staged_smem_bytes<MODEL, DAMP>(), stream>>>(sp);
    return cudaPeekAtLastError();
}

int staged_test_hold(int plane, int polls)
{
    const int h = plane >= 0 ? plane : -1;
    const int v = (plane >= 0 && polls > 0) ? polls : kStagedWaitPolls;
    if (cudaMemcpyToSymbol(g_staged_wait_limit, &v, sizeof(int)) != cudaSuccess) return -1;
    if (cudaMemcpyToSymbol(g_staged_hold, &h, sizeof(int)) != cudaSuccess) return -1;
    return 0;
}

bool staged_take_error()
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_staged_err, sizeof(int)) != cudaSuccess) return true;
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_staged_err, &zero, sizeof(int));
    }
    return v != 0;
}

#define EWF_STAGED_INSTANCE(MODEL, DAMP)                                                                   \
    template bool staged_ready<MODEL, DAMP>();                                                           \
    template cudaError_t staged_launch<MODEL, DAMP>(const FusedArgs<float> &, const StagedPlan &, int, int, cudaStream_t);
EWF_STAGED_INSTANCE(MODEL_ISO, DAMP_PML1D)
EWF_STAGED_INSTANCE(MODEL_ORTHO, DAMP_W3D)
EWF_STAGED_INSTANCE(MODEL_ORTHO, DAMP_SEP)
#undef EWF_STAGED_INSTANCE

}  // namespace ewf
