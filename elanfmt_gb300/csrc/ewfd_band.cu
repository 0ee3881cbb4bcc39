// ewfd_band.cu -- instances and launches of the band form of the one-pass step (ewfd_band.cuh).
#include "ewfd_band.cuh"

namespace ewf {

template <typename T, int MODEL, int DAMP, bool KAHAN, int BY>
static cudaLaunchConfig_t band_config(dim3 grid, cudaStream_t stream, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(BX, BY, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = grid.x;  // one cluster spans the band
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <typename T, int MODEL, int DAMP, bool KAHAN, int BY>
static cudaError_t clusters_rows(dim3 grid, int *clusters)
{
    *clusters = 0;
    if (grid.x < 1 || grid.x > (unsigned)BAND_MAX_CTAS) return cudaSuccess;
    auto kern = k_band<T, MODEL, DAMP, KAHAN, BY>;
    if (grid.x > 8) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = band_config<T, MODEL, DAMP, KAHAN, BY>(grid, nullptr, attr);
    return cudaOccupancyMaxActiveClusters(clusters, kern, &cfg);
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
cudaError_t band_clusters(int rows, dim3 grid, int *clusters)
{
    if constexpr (sizeof(T) == 4) {
        if (rows == 8) return clusters_rows<T, MODEL, DAMP, KAHAN, 8>(grid, clusters);
    }
    if (rows == 4) return clusters_rows<T, MODEL, DAMP, KAHAN, 4>(grid, clusters);
    *clusters = 0;
    return cudaErrorInvalidValue;
}

template <typename T, int MODEL, int DAMP, bool KAHAN, int BY>
static cudaError_t launch_rows(const FusedArgs<T> &fa, dim3 grid, cudaStream_t stream)
{
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = band_config<T, MODEL, DAMP, KAHAN, BY>(grid, stream, attr);
    return cudaLaunchKernelEx(&cfg, k_band<T, MODEL, DAMP, KAHAN, BY>, fa);
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
cudaError_t band_launch(const FusedArgs<T> &fa, int rows, dim3 grid, cudaStream_t stream)
{
    if constexpr (sizeof(T) == 4) {
        if (rows == 8) return launch_rows<T, MODEL, DAMP, KAHAN, 8>(fa, grid, stream);
    }
    if (rows == 4) return launch_rows<T, MODEL, DAMP, KAHAN, 4>(fa, grid, stream);
    return cudaErrorInvalidValue;
}

// the combinations the one-pass form is built for (models 0 and 1; 1-D PML for the isotropic
// scheme, 3-D or separable weights for the orthorhombic one; FP32, Kahan FP32, FP64)
#define EWF_BAND_INSTANCE(T, MODEL, DAMP, KAHAN)                                                              \
    template cudaError_t band_clusters<T, MODEL, DAMP, KAHAN>(int, dim3, int *);                             \
    template cudaError_t band_launch<T, MODEL, DAMP, KAHAN>(const FusedArgs<T> &, int, dim3, cudaStream_t);
EWF_BAND_INSTANCE(float, MODEL_ISO, DAMP_PML1D, false)
EWF_BAND_INSTANCE(float, MODEL_ORTHO, DAMP_W3D, false)
EWF_BAND_INSTANCE(float, MODEL_ORTHO, DAMP_SEP, false)
EWF_BAND_INSTANCE(float, MODEL_ISO, DAMP_PML1D, true)
EWF_BAND_INSTANCE(float, MODEL_ORTHO, DAMP_W3D, true)
EWF_BAND_INSTANCE(float, MODEL_ORTHO, DAMP_SEP, true)
EWF_BAND_INSTANCE(double, MODEL_ISO, DAMP_PML1D, false)
EWF_BAND_INSTANCE(double, MODEL_ORTHO, DAMP_W3D, false)
EWF_BAND_INSTANCE(double, MODEL_ORTHO, DAMP_SEP, false)
#undef EWF_BAND_INSTANCE

}  // namespace ewf
