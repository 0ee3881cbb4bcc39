// ewf_umma.h -- operand layout and descriptors of the surrogate's tcgen05 (UMMA) GEMM
// (host and device code; the host side is exercised by tests/test_umma_layout_cpu.py).
//
// One CTA computes a BM x BN tile of C = A . B^T with A [M, K] and B [N, K] both K-major bf16.
// A k-stage of BK = 64 elements (128 bytes of every operand row) is brought into shared memory
// by one 2-D TMA copy per operand with the 128-byte swizzle: row r of a stage tile occupies bytes
// [r * 128, r * 128 + 128) and its 16-byte chunk c sits at chunk c ^ (r % 8).  That is the
// tensor core's canonical K-major SWIZZLE_128B layout: 8-row atoms of 1024 bytes, one after the
// other (stride-dimension offset 1024 B), and the k-th MMA of a stage (K = 16, 32 bytes of each
// row) starts its descriptors 32 k bytes into the atom.  Stage tiles start on 1024-byte
// boundaries, so the descriptors' base offset is 0.
//
// Shared-memory matrix descriptor (64 bit): start address >> 4 in bits 0-13, leading-dimension
// byte offset >> 4 in bits 16-29 (not used by swizzled K-major layouts; 16 B), stride-dimension
// byte offset >> 4 in bits 32-45, descriptor version 1 in bits 46-47, base offset 0 (bits
// 49-51), layout type in bits 61-63 (2 = SWIZZLE_128B).
// Instruction descriptor (32 bit, kind::f16): D format F32 (1) in bits 4-5, A and B format BF16
// (1) in bits 7-9 and 10-12, both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in
// bits 24-28.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define EWF_UHD __host__ __device__ __forceinline__
#else
#define EWF_UHD inline
#endif

namespace ewf_umma {

constexpr int BM = 128;          // rows of A per CTA tile (TMEM lanes of the accumulator)
constexpr int BK = 64;           // K per pipeline stage: 128 bytes per operand row
constexpr int STAGES = 4;
constexpr int ROW_BYTES = BK * 2;
constexpr int ATOM_BYTES = 8 * ROW_BYTES;  // 8 rows x 128 B: the swizzle atom, stride-dimension offset
constexpr int MMA_K = 16;
constexpr int THREADS = 192;     // warp 0: TMA producer (one lane); warp 1: MMA issuer (one lane); warps 2-5: epilogue
constexpr int LAYOUT_SW128 = 2;

// Per tile width BN (128 or 256): bytes of a stage and of the whole pipeline; TMEM columns = 2 BN
// (two accumulators).
EWF_UHD constexpr int a_bytes() { return BM * ROW_BYTES; }
EWF_UHD constexpr int b_bytes(int bn) { return bn * ROW_BYTES; }
EWF_UHD constexpr int stage_bytes(int bn) { return a_bytes() + b_bytes(bn); }
EWF_UHD constexpr int smem_bytes(int bn) { return STAGES * stage_bytes(bn) + 1024; }  // + alignment slack

EWF_UHD uint64_t smem_desc_sw128(uint32_t smem_addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((smem_addr >> 4) & 0x3FFFu);
    d |= (uint64_t)(16 >> 4) << 16;
    d |= (uint64_t)((ATOM_BYTES >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // version
    d |= (uint64_t)LAYOUT_SW128 << 61;
    return d;
}

EWF_UHD uint32_t instr_desc_bf16_f32(int m, int n)
{
    uint32_t d = 0;
    d |= 1u << 4;   // D: F32
    d |= 1u << 7;   // A: BF16
    d |= 1u << 10;  // B: BF16
    d |= (uint32_t)((n >> 3) & 0x3F) << 17;
    d |= (uint32_t)((m >> 4) & 0x1F) << 24;
    return d;
}

// The end of the byte range an MMA of a stage reads from one operand tile of `rows` rows: every
// 8-row atom from the start address (32 k bytes into the first row) on, to the end of the last
// row's 32-byte K slice.
EWF_UHD uint32_t mma_read_end(uint32_t start, int rows)
{
    return start + (uint32_t)(rows / 8 - 1) * ATOM_BYTES + 7 * ROW_BYTES + 32;
}

// Phase bookkeeping of the GEMM's mbarriers.  An mbarrier wait with parity P returns once the
// barrier's current phase has a parity other than P, i.e. once the latest completed phase has
// parity P; a fresh barrier (phase 0 running) therefore lets a parity-1 wait through at once.
// Stage ring: the g-th k-stage of a CTA (counted across its tiles) uses slot g % STAGES; its
// "full" completion is that slot's (g / STAGES)-th, its "empty" completion frees the slot for
// stage g + STAGES.  Accumulators: the i-th tile of a CTA uses buffer i % 2; "acc_full" completes
// once per tile in that buffer, "acc_empty" once per drained tile.
EWF_UHD int ring_slot(int g) { return g % STAGES; }
EWF_UHD uint32_t ring_full_parity(int g) { return (uint32_t)(g / STAGES) & 1u; }          // consumer of stage g
EWF_UHD bool ring_needs_free(int g) { return g >= STAGES; }                               // producer of stage g waits?
EWF_UHD uint32_t ring_free_parity(int g) { return (uint32_t)(g / STAGES - 1) & 1u; }     // ... for stage g - STAGES
EWF_UHD int acc_buf(int i) { return i & 1; }
EWF_UHD uint32_t acc_full_parity(int i) { return (uint32_t)(i >> 1) & 1u; }              // epilogue of tile i
EWF_UHD bool acc_needs_free(int i) { return i >= 2; }                                     // MMAs of tile i wait?
EWF_UHD uint32_t acc_free_parity(int i) { return (uint32_t)((i >> 1) - 1) & 1u; }        // ... for tile i - 2

}  // namespace ewf_umma
