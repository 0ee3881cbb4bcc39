// ewfd_band.h -- host interface of the band form of the one-pass step (kernel: ewfd_band.cuh,
// instances and launches: ewfd_band.cu).
#pragma once
#include <cuda_runtime.h>

#include "ewfd_fused.cuh"

namespace ewf {

constexpr int BX = 64;             // band CTA width in columns (two warps per row)
constexpr int BAND_MAX_CTAS = 16;  // CTAs per cluster = ceil(nx / BX) (above 8: non-portable cluster size)

// Grid of the band kernel: x = the band's CTAs (one cluster), y = bands of `rows` rows, z = z-chunks.
inline dim3 band_grid(int nx, int ny, int nz, int rows, int kchunk)
{
    return dim3((unsigned)((nx + BX - 1) / BX), (unsigned)((ny + rows - 1) / rows), (unsigned)((nz + kchunk - 1) / kchunk));
}

// Is `rows` a band height built for this element type (4 or 8 rows in FP32, 4 in FP64)?
template <typename T>
inline bool band_rows_built(int rows) { return rows == 4 || (rows == 8 && sizeof(T) == 4); }

// Clusters of the band kernel that fit on the current device at once (0: it cannot run there);
// allows the non-portable cluster size first where the band needs more than 8 CTAs.
template <typename T, int MODEL, int DAMP, bool KAHAN>
cudaError_t band_clusters(int rows, dim3 grid, int *clusters);

// One launch of the band kernel (one time step; grid from band_grid).
template <typename T, int MODEL, int DAMP, bool KAHAN>
cudaError_t band_launch(const FusedArgs<T> &fa, int rows, dim3 grid, cudaStream_t stream);

}  // namespace ewf
