// Host check of the tcgen05 GEMM's stage layout and descriptors (elanfmt_gb300/csrc/ewf_umma.h),
// compiled with g++ by tests/test_umma_layout_cpu.py, for both tile widths (BN = 128, 256):
//   1. the pipeline fits in shared memory and every stage tile starts on a 1024-byte boundary
//      (the 128-byte swizzle's atom; the descriptors' base offset is 0);
//   2. the bytes a stage's TMA boxes deliver (BK x rows bf16 per operand) equal the stage size
//      the "full" barrier expects;
//   3. every byte range an MMA of the stage reads (8-row atoms from its start, 32 k bytes into
//      the first row) lies inside its operand tile;
//   4. the descriptor fields decode back to their inputs (start address, offsets, version,
//      SWIZZLE_128B) and the instruction descriptor holds M = 128, N = BN, BF16 / BF16 -> F32;
//   5. the two accumulators' 2 x BN fp32 columns are a legal tensor-memory allocation.
// Prints "ok" or the first failure.
#include <cstdio>

#include "ewf_umma.h"

using namespace ewf_umma;

static int fail(const char *what, long a, long b)
{
    printf("FAIL %s %ld %ld\n", what, a, b);
    return 1;
}

static int check(int bn)
{
    if (smem_bytes(bn) > 227 * 1024) return fail("smem", bn, smem_bytes(bn));
    for (int s = 0; s < STAGES; ++s) {
        const int a = s * stage_bytes(bn), b = a + a_bytes();
        if (a % 1024 || b % 1024) return fail("stage alignment", bn, s);
        if (b + b_bytes(bn) > STAGES * stage_bytes(bn)) return fail("stage range", bn, s);
    }
    if (BK * 2 * (BM + bn) != stage_bytes(bn)) return fail("tma bytes vs expect_tx", bn, stage_bytes(bn));
    if (ROW_BYTES != 128) return fail("box inner bytes must equal the swizzle span", ROW_BYTES, 128);
    for (int j = 0; j < BK / MMA_K; ++j) {
        if (mma_read_end(32 * j, BM) > (uint32_t)a_bytes()) return fail("A read past the tile", bn, j);
        if (mma_read_end(32 * j, bn) > (uint32_t)b_bytes(bn)) return fail("B read past the tile", bn, j);
    }
    const uint32_t id = instr_desc_bf16_f32(BM, bn);
    if (((id >> 4) & 3) != 1 || ((id >> 7) & 7) != 1 || ((id >> 10) & 7) != 1) return fail("idesc formats", id, 0);
    if (((id >> 13) & 0xF) != 0) return fail("idesc negate / major", id, 0);
    if ((int)((id >> 17) & 0x3F) != bn / 8 || (int)((id >> 24) & 0x1F) != BM / 16) return fail("idesc shape", id, bn);
    if (id & ((1u << 23) | (1u << 29) | 0xFu | (3u << 30) | (1u << 6))) return fail("idesc reserved bits", id, 0);
    const int cols = 2 * bn;
    if (cols < 32 || (cols & (cols - 1)) || cols > 512) return fail("tmem columns", cols, 0);
    if (THREADS != 192) return fail("warp roles: 1 producer + 1 MMA + 4 epilogue warps", THREADS, 192);
    return 0;
}

int main()
{
    if (check(128) || check(256)) return 1;
    const uint32_t addr = 0x2A400;  // a 1024-byte aligned shared address below 256 KB
    const uint64_t d = smem_desc_sw128(addr + 64);
    if ((d & 0x3FFF) != ((addr + 64) >> 4)) return fail("desc start", (long)(d & 0x3FFF), (addr + 64) >> 4);
    if (((d >> 16) & 0x3FFF) != 1) return fail("desc lbo", (long)((d >> 16) & 0x3FFF), 1);
    if (((d >> 32) & 0x3FFF) != ATOM_BYTES >> 4) return fail("desc sbo", (long)((d >> 32) & 0x3FFF), ATOM_BYTES >> 4);
    if (((d >> 46) & 3) != 1) return fail("desc version", (long)((d >> 46) & 3), 1);
    if ((d >> 49) & 0xF) return fail("desc base offset / lbo mode", (long)((d >> 49) & 0xF), 0);
    if ((d >> 61) != (uint64_t)LAYOUT_SW128) return fail("desc layout", (long)(d >> 61), LAYOUT_SW128);
    if ((smem_desc_sw128(0x3FFF0) & 0x3FFF) != 0x3FFF) return fail("desc start width", 0, 0);
    printf("ok\n");
    return 0;
}
