// ewfd_batch.cuh -- batched time step: many problems (models of uneven size) x many right-hand
// sides (sources) advanced together.
//
// A problem is one model (grid, materials, damping) with R right-hand sides (source sets); its R
// state sets are separate boxes (rhs_stride elements apart) sharing the material arrays.
// * Problems with several RHS (k_stress_mr / k_velocity_mr) get a launch of their own whose
//   blockIdx.x runs over (x-tile, RHS) with the RHS fastest: the R CTAs that update one tile for
//   the R right-hand sides are dispatched together, so the tile's material planes come from HBM
//   once and from L2 for the other R-1 (the 6 elementary moment tensors of a moment-tensor
//   inversion share one model).
// * Single-RHS problems of one (model, damping) family share one persistent launch (k_bstress /
//   k_bvelocity): the grid is sized to the GPU and each CTA strides over a work list of
//   (problem, z-chunk, y-tile, x-tile) items, so models of very different sizes share one launch
//   without a tail per problem.
// Every item is the single-problem column update (stress_column / velocity_column).
#pragma once
#include "ewfd_fused.cuh"

namespace ewf {

template <typename T>
struct BatchProb {
    StepArgs<T> a;                        // the problem, state of RHS 0
    long long rhs_stride;                 // elements between the state boxes of consecutive RHS
    int R, tiles_x, tiles_y, chunks, item0;  // work items of this problem start at item0
};

// CTAs are TX x blockDim.y columns; blockDim.y (the tile height, autotuned) is one of 4, 8, 16.
constexpr int BATCH_MIN_TY = 4;
constexpr int BATCH_MAX_TY = 16;

__device__ __forceinline__ int find_problem(const int *item0, int nprob, int item)
{
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (item0[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Stages the StepArgs of the item's RHS in shared memory (so the column routine reads its fields
// from there instead of pinning ~40 of them in registers) and returns the column coordinates.
template <typename T>
__device__ __forceinline__ void item_args(const BatchProb<T> &P, int item, StepArgs<T> &sa, int &X, int &j, int &k0,
                                          int &k1)
{
    int rem = item - P.item0;
    const int r = rem % P.R;
    rem /= P.R;
    const int tx_ = rem % P.tiles_x;
    rem /= P.tiles_x;
    const int ty_ = rem % P.tiles_y;
    const int ch = rem / P.tiles_y;
    X = tx_ * TX + threadIdx.x;
    j = ty_ * (int)blockDim.y + threadIdx.y;
    k0 = ch * P.a.kchunk;
    k1 = min(k0 + P.a.kchunk, P.a.nz);
    __syncthreads();  // the previous item is done with sa
    const int t = threadIdx.y * TX + threadIdx.x;
    constexpr int NW = sizeof(StepArgs<T>) / sizeof(int);
    static_assert(sizeof(StepArgs<T>) % sizeof(int) == 0, "StepArgs is copied as words");
    static_assert(NW <= TX * BATCH_MIN_TY, "the smallest CTA copies StepArgs in one pass");
    if (t < NW) reinterpret_cast<int *>(&sa)[t] = reinterpret_cast<const int *>(&P.a)[t];
    __syncthreads();
    if (t < 9) sa.f[t] += (long long)r * P.rhs_stride;
    __syncthreads();
}

// Stress phase for every problem of one (model, damping) family: a persistent grid striding
// over the work items.
template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(TX * BATCH_MAX_TY, 2) k_bstress(const BatchProb<T> *__restrict__ probs,
                                                         const int *__restrict__ item0, int nprob, int nitems)
{
    __shared__ StepArgs<T> sa;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int pid = find_problem(item0, nprob, item);
        int X, j, k0, k1;
        item_args(probs[pid], item, sa, X, j, k0, k1);
        stress_column<T, MODEL, DAMP, 1>(sa, X, j, k0, k1);
    }
}

template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(TX * BATCH_MAX_TY, 2) k_bvelocity(const BatchProb<T> *__restrict__ probs,
                                                           const int *__restrict__ item0, int nprob, int nitems)
{
    __shared__ StepArgs<T> sa;
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int pid = find_problem(item0, nprob, item);
        int X, j, k0, k1;
        item_args(probs[pid], item, sa, X, j, k0, k1);
        velocity_column<T, MODEL, DAMP, false, 1>(sa, X, j, k0, k1);
    }
}

// One problem with R right-hand sides in separate boxes (rhs_stride elements apart), launched on
// its own: the problem's arguments stay in the kernel's parameter space (read by the column code
// as constant-bank operands, as in k_stress), the RHS index is the fastest part of blockIdx.x,
// so the R CTAs of a tile are dispatched together and read the tile's material planes from HBM
// once (the other R-1 reads hit L2).
template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(TX * BATCH_MAX_TY, 2) k_stress_mr(const StepArgs<T> a, int R, long long rhs_stride)
{
    const int r = blockIdx.x % R;
    const int tx = blockIdx.x / R;
    const int k0 = blockIdx.z * a.kchunk;
    stress_column<T, MODEL, DAMP, 1, true>(a, tx * TX + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y, k0,
                                        min(k0 + a.kchunk, a.nz), (long long)r * rhs_stride);
}

template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(TX * BATCH_MAX_TY, 2) k_velocity_mr(const StepArgs<T> a, int R, long long rhs_stride)
{
    const int r = blockIdx.x % R;
    const int tx = blockIdx.x / R;
    const int k0 = blockIdx.z * a.kchunk;
    // REC: the L2 prefetch of the state inputs a.l2pf planes ahead (no receivers: col_first is null)
    velocity_column<T, MODEL, DAMP, false, 1, true, 0, true>(a, tx * TX + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y,
                                                          k0, min(k0 + a.kchunk, a.nz), (long long)r * rhs_stride, RecFuse{});
}

// Point injection for every (problem, RHS): one thread per (problem, RHS), entries in order,
// with the same before/after-BC1 semantics as k_inject.
struct BatchSrc {
    int prob, rhs, comp, i, j, k;
    double coef;
};

template <typename T>
__global__ void k_binject(const BatchProb<T> *__restrict__ probs, const BatchSrc *__restrict__ src,
                          const int *__restrict__ src_start, int ngroups, const double *__restrict__ stf,
                          const int *__restrict__ stf_off, const int *__restrict__ order, int nstf,
                          const int *__restrict__ it_ptr)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    const int it = *it_ptr;
    if (it < 0 || it >= nstf) return;
    for (int e = src_start[g]; e < src_start[g + 1]; ++e) {
        const BatchSrc q = src[e];
        const StepArgs<T> &P = probs[q.prob].a;
        const T s = (T)stf[stf_off[q.prob] + it];
        const long long c = (long long)q.i + (long long)q.j * P.sx + (long long)q.k * P.sy + (long long)q.rhs * probs[q.prob].rhs_stride;
        T *f = P.f[q.comp];
        if (order[q.prob] == 0) {
            const bool row_bc = q.j < P.bc1_rows;
            const bool xz_bc = (q.comp == 7) && q.i > 0 && q.i < P.nx && row_bc;
            const bool yz_bc = (q.comp == 8) && q.j > 0 && q.j < P.ny && q.i < P.nx;
            if ((q.comp == 5 && q.k == 0 && row_bc) || ((xz_bc || yz_bc) && q.k == 1)) continue;
            f[c] = f[c] + (T)q.coef * s;
            if ((xz_bc || yz_bc) && q.k == 2) f[c - P.sy] = P.third * f[c];
        } else {
            f[c] = f[c] + (T)q.coef * s;
        }
    }
}

// Receiver gather for every problem and RHS; advances the batch step counter.
template <typename T>
__global__ void k_brecord(const BatchProb<T> *__restrict__ probs, const int *__restrict__ rec_prob,
                          const long long *__restrict__ rec_off, const int *__restrict__ rec_comp, int nrec,
                          double *__restrict__ traces, int nt, int *it_ptr)
{
    // traces[r * nt + it], where r runs over (receiver, rhs) pairs in the order the host built
    const int it = *it_ptr;
    if (it >= 0 && it < nt)
        for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
            const StepArgs<T> &P = probs[rec_prob[r]].a;
            traces[(long long)r * nt + it] = (double)P.f[rec_comp[r]][rec_off[r]];
        }
}

__global__ void k_advance(int *it_ptr) { *it_ptr += 1; }

}  // namespace ewf
