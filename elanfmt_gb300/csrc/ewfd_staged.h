// ewfd_staged.h -- host interface of the staged form of the one-pass step (kernel: ewfd_staged.cuh,
// instances, tensor maps and launches: ewfd_staged.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "ewfd_fused.cuh"

namespace ewf {

constexpr int SX = 64;                 // tile width (two warps per row)
constexpr int SY = 8;                  // tile height
constexpr int SHX = 4;                 // x halo of a staged box: 16-byte aligned start for TMA
constexpr int SBW = SX + 2 * SHX;      // staged box width: columns i0-4 .. i0+SX+3
constexpr int SBH = SY + 2;            // staged box height: rows j0-1 .. j0+SY
constexpr int SBOX = 736;              // floats per staged field: SBW * SBH = 720, padded to 128 bytes
constexpr int SOWN = SX * SY;          // floats per own-box field (buoyancy)
constexpr int SNSTAGE = 3;             // planes in the ring (two in flight while one is read)

// Tensor maps of one launch: the state read this step (9 fields), the moduli and 3-D weight (up to
// 10) in boxes of SBW x SBH x 1 around the tile, the buoyancy (3) in boxes of SX x SY x 1.
struct StagedMaps {
    CUtensorMap st[9];
    CUtensorMap mt[10];
    CUtensorMap bu[3];
};

// Per handle: the maps of both state buffers (parity 0: f_alloc read, 1: g_alloc read).
struct StagedPlan {
    StagedMaps maps[2];
    bool ok = false;
};

// Encodes the tensor maps of a handle's allocations (3-D boxes over its padded geometry: sx x
// (ny + 3) x (nz + 3) floats, the allocation starting at element (-hx, -1, -1)).  Returns false
// when the driver's encoder is unavailable or rejects a map.
bool staged_encode(StagedPlan &plan, void *const f_alloc[9], void *const g_alloc[9], void *const m_alloc[12],
                   void *w3_alloc, int nmat_big, const int *mat_slots, bool w3, bool buoyancy, int sx, int ny, int nz);

// Can the staged kernel run on the current device (its shared memory fits)?  Sets the kernel's
// shared-memory attribute on first use per device.
template <int MODEL, int DAMP>
bool staged_ready();

// One launch (one time step) reading the state of `parity` (hx: element offset of i = 0 in an
// allocation's rows).  Launch errors are left for the caller's cudaGetLastError.
template <int MODEL, int DAMP>
cudaError_t staged_launch(const FusedArgs<float> &fa, const StagedPlan &plan, int parity, int hx, cudaStream_t stream);

// Reads and clears the staged kernel's error flag (a bounded wait for a plane stage gave up, so
// the state written by that run is invalid).  Call after the stream has been synchronised.
bool staged_take_error();

// Test hook (ewf_staged_test_hold): the first CTA never issues the copies of plane `plane` and
// every wait gives up after `polls` polls; plane < 0 restores normal operation.  0 or -1 (CUDA error).
int staged_test_hold(int plane, int polls);

}  // namespace ewf
