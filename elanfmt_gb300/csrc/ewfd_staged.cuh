// ewfd_staged.cuh -- one-pass time step over tiles whose planes are staged in shared memory by TMA.
//
// The tile and band kernels of the one-pass step spend most of their instructions on addresses:
// with runtime row and plane pitches every neighbour load needs its own 64-bit address (361 of
// the band kernel's 816 instructions per cell were integer).  k_staged moves the data with the
// tensor memory accelerator instead:
//   * state is double-buffered as in k_step (step n read, step n+1 written);
//   * a CTA owns a 64 x 8 column tile and marches its z-chunk; one thread issues, two planes
//     ahead, one 3-D TMA copy per field and plane into a ring of three plane stages: every state
//     field, modulus and 3-D weight as a box of columns i0-4 .. i0+67 and rows j0-1 .. j0+8 (the
//     tile with the halo its stencils read; x starts on a 16-byte boundary), the buoyancy as the
//     64 x 8 tile of the plane below (the velocity update's plane); each stage's copies complete
//     on its mbarrier (bounded waits; a wait that gives up raises an error flag the host reads);
//   * threads read their stencils from the stage at compile-time offsets, compute sigma(p) and
//     stage the five components with x/y neighbours (own cells plus the ring the velocity update
//     reads: sxx at i0-1, syy at j0-1, sxy at i0+64 and j0+8, sxz at i0+64, syz at j0+8, recomputed
//     by nine warps from the same stage) in one of three buffers, then after one CTA barrier
//     update V(p-1); the own column's V(p-1) and szz(p-1..p-2) stay in registers;
//   * every read of a plane stage happens before the plane's barrier, so the stage can be
//     refilled (with plane p+3) right after it; the stress buffers rotate over three planes, so one
//     barrier per plane guards both;
//   * BC1 (OK4:271-283) and the moment-tensor injection in both reference orders (OK4:336-342
//     before BC1, ANISO:533-535 after) are replayed as in k_step, with the same arithmetic.
// FP32 without compensation; the orthorhombic model with 3-D or separable weights and the
// isotropic model with 1-D PML profiles.
#pragma once
#include "ewfd_band.cuh"  // HaloConst, halo_const
#include "ewfd_staged.h"

namespace ewf {

__device__ int g_staged_err = 0;
constexpr int kStagedWaitPolls = 1 << 22;
__device__ int g_staged_wait_limit = kStagedWaitPolls;  // polls before a wait gives up
__device__ int g_staged_hold = -1;  // test hook: plane whose copies the first CTA never issues (-1: none)

__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void st_mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool st_mbar_try(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
// Bounded wait for a plane stage (limit: g_staged_wait_limit, read once per launch); gives up at
// once when another wait has already given up.
__device__ __forceinline__ bool st_mbar_wait(unsigned bar, unsigned parity, int limit)
{
    for (int n = 0; n < limit; ++n) {
        if (st_mbar_try(bar, parity)) return true;
        if ((n & 1023) == 1023 && *(volatile int *)&g_staged_err) return false;
    }
    atomicExch(&g_staged_err, 1);
    return false;
}
__device__ __forceinline__ void st_mbar_expect(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void st_tma3(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

template <int MODEL, int DAMP>
struct StagedLayout {
    static constexpr int NC = MODEL == MODEL_ISO ? 2 : 9;                       // moduli
    static constexpr int NW = (MODEL != MODEL_ISO && DAMP == DAMP_W3D) ? 1 : 0;  // 3-D weight
    static constexpr int NBIG = 9 + NC + NW;                                    // boxes around the tile
    static constexpr int NB = MODEL == MODEL_ISO ? 0 : 3;                       // buoyancy tiles
    static constexpr int STAGE_FLOATS = NBIG * SBOX + NB * SOWN;
    static constexpr unsigned TX_BYTES = (unsigned)(NBIG * SBW * SBH + NB * SOWN) * 4u;
};

// The stresses staged for the velocity update, one plane (layout as in k_band with BX = 64, BY = 8).
struct StagedStress {
    float xx[SY][SX + 1];      // own at [ty][tx + 1]; col 0: i0-1
    float yy[SY + 1][SX];      // own at [ty + 1][tx]; row 0: j0-1
    float xy[SY + 1][SX + 1];  // own at [ty][tx]; row SY: j0+SY; col SX: i0+SX
    float xz[SY][SX + 1];      // own at [ty][tx]; col SX: i0+SX
    float yz[SY + 1][SX];      // own at [ty][tx]; row SY: j0+SY
};

// Dynamic shared memory: the plane stages, three stress buffers, the mbarriers, the source list.
constexpr size_t STG_BYTES = (sizeof(StagedStress) + 127) / 128 * 128;
template <int MODEL, int DAMP>
__host__ __device__ constexpr size_t staged_stage_bytes() { return (size_t)SNSTAGE * StagedLayout<MODEL, DAMP>::STAGE_FLOATS * 4; }
template <int MODEL, int DAMP>
__host__ __device__ constexpr size_t staged_smem_bytes()
{
    return staged_stage_bytes<MODEL, DAMP>() + 3 * STG_BYTES + 4 * 8 + MAXSRC * sizeof(SrcEntry) + 16 + 128;  // + 128: base alignment
}

struct StagedParams {
    FusedArgs<float> fa;
    StagedMaps maps;
    int hx;  // element offset of i = 0 in an allocation's rows
};

// One stress component (4 syy, 6 sxy, 7 sxz, 8 syz, 3 sxx) of step n+1 at the staged position hb
// (cell (i, j), plane p): halo_sigma's arithmetic on the staged plane (Sp), the next plane's Vz
// (Sn) and vm, the own position's Vx (comp 7) or Vy (comp 8) on plane p-1; 0 where the reference
// does not update the cell.
template <int MODEL, int DAMP>
__device__ __forceinline__ float staged_sigma(const StepArgs<float> &a, int comp, int i, int j, int p, int hb,
                                              const float *Sp, const float *Sn, float vm, const HaloConst<float> &hk,
                                              float wz)
{
    using L = StagedLayout<MODEL, DAMP>;
    const int nx = a.nx, ny = a.ny;
    bool upd;
    if (comp == 3 || comp == 4 || MODEL == MODEL_ISO) upd = (i >= 0 && j >= 0 && i < nx && j < ny);
    else if (comp == 6) upd = (i > 0 && j > 0 && i < nx && j < ny);
    else if (comp == 7) upd = (i > 0 && i < nx && j >= 0 && j < ny && p > 0);
    else upd = (j > 0 && j < ny && i >= 0 && i < nx && p > 0);
    if (!upd) return 0.f;
    const float *Vx = Sp, *Vy = Sp + SBOX, *Vz = Sp + 2 * SBOX, *C = Sp + 9 * SBOX;
    const float dt = a.dt, old = Sp[comp * SBOX + hb];
    float W = 0.f;
    if (MODEL != MODEL_ISO) W = (DAMP == DAMP_W3D) ? Sp[(9 + L::NC) * SBOX + hb] : hk.pxy * wz;
    if (comp == 3 || comp == 4) {
        const float Vxx = (Vx[hb + 1] - Vx[hb]) * a.rdx;
        const float Vyy = (Vy[hb + SBW] - Vy[hb]) * a.rdy;
        const float Vzz = (Sn[2 * SBOX + hb] - Vz[hb]) * a.rdz;
        if (MODEL == MODEL_ISO) {
            const float c11 = C[hb], c12 = C[SBOX + hb];
            if (comp == 3) return nrm_iso(hk.wav, old, dt, c11, c12, c12, Vxx, Vyy, Vzz);
            return nrm_iso(hk.wav, old, dt, c12, c11, c12, Vxx, Vyy, Vzz);
        }
        if (comp == 3) return nrm_ortho(old, W, dt, C[hb], C[3 * SBOX + hb], C[4 * SBOX + hb], Vxx, Vyy, Vzz);
        return nrm_ortho(old, W, dt, C[3 * SBOX + hb], C[SBOX + hb], C[5 * SBOX + hb], Vxx, Vyy, Vzz);
    }
    float d1, d2;
    if (comp == 6) {
        d1 = Vy[hb] - Vy[hb - 1];
        d2 = Vx[hb] - Vx[hb - SBW];
    } else if (comp == 7) {
        d1 = Vz[hb] - Vz[hb - 1];
        d2 = Vx[hb] - vm;
    } else {
        d1 = Vy[hb] - vm;
        d2 = Vz[hb] - Vz[hb - SBW];
    }
    if (MODEL == MODEL_ISO) {
        const float wx = hk.wx, wy = hk.wy;
        const float c66dt = a.c66 * dt;
        if (comp == 6) return shr_iso(wz * wy * wx, old, c66dt, d1, a.rdx, d2, a.rdy);
        if (comp == 7) return shr_iso(wy * wz * wx, old, c66dt, d1, a.rdx, d2, a.rdz);
        return shr_iso(wx * wy * wz, old, c66dt, d1, a.rdz, d2, a.rdy);
    }
    if (comp == 6) return shr_ortho(old, W, dt, C[6 * SBOX + hb], d1, a.dx, a.rdx, d2, a.dy, a.rdy, a.fdiv != 0);
    if (comp == 7) return shr_ortho(old, W, dt, C[7 * SBOX + hb], d1, a.dx, a.rdx, d2, a.dz, a.rdz, a.fdiv != 0);
    return shr_ortho(old, W, dt, C[8 * SBOX + hb], d1, a.dz, a.rdz, d2, a.dy, a.rdy, a.fdiv != 0);
}

template <int MODEL, int DAMP>
__global__ void __launch_bounds__(SX *SY, 1) k_staged(const __grid_constant__ StagedParams sp)
{
    using T = float;
    using L = StagedLayout<MODEL, DAMP>;
    const FusedArgs<T> &fa = sp.fa;
    const StepArgs<T> &a = fa.a;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_raw + ((128u - (su32(smem_raw) & 127u)) & 127u);
    float *stages = reinterpret_cast<float *>(smem);
    unsigned char *stg_base = smem + staged_stage_bytes<MODEL, DAMP>();
    auto stg = [&](int q) -> StagedStress & { return *reinterpret_cast<StagedStress *>(stg_base + q * STG_BYTES); };
    unsigned long long *full = reinterpret_cast<unsigned long long *>(stg_base + 3 * STG_BYTES);
    SrcEntry *s_src = reinterpret_cast<SrcEntry *>(full + 4);
    int *s_nsrc = reinterpret_cast<int *>(s_src + MAXSRC);

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * SX + tx, warp = tid >> 5, lane = tid & 31;
    const int i0 = blockIdx.x * SX, j0 = blockIdx.y * SY;
    const int i = i0 + tx, j = j0 + ty;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int k0 = blockIdx.z * a.kchunk;
    const int k1 = min(k0 + a.kchunk, nz);
    const int ps = (k0 == 0) ? 0 : k0 - 1;
    const int plast = k1 + 1;  // planes ps .. k1 + 1 are staged (Vz(k1 + 1) for sigma(k1))
    const int sx = a.sx;
    const long long sy = a.sy;
    const T dt = a.dt, rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;
    const bool in_grid = (i < nx && j < ny);
    const bool row_bc = (j < a.bc1_rows);

    // plane q into stage q % 3 (thread 0)
    // the test hook and the wait limit, read once (they do not change during a launch)
    const int wait_limit = *(volatile int *)&g_staged_wait_limit;
    const int held_plane = (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) ? *(volatile int *)&g_staged_hold : -1;
    // thread 0's record of the fills it issued per stage (each completes one mbarrier phase): bit s
    // of filled = at least one, of odd = an odd number; waits_ok = none of its waits gave up
    unsigned filled = 0, odd = 0;
    bool waits_ok = true;
    // the last fill of stage s has landed (bounded wait on its phase)
    auto drain_stage = [&](int s) {
        const unsigned par = ((odd >> s) & 1u) ^ 1u;
        for (int n = 0; n < wait_limit; ++n)
            if (st_mbar_try(su32(&full[s]), par)) break;
    };
    auto issue = [&](int q) {
        if (q == held_plane) return;  // test hook: a fill nothing completes
        const int s = q % SNSTAGE;
        // never two fills of one stage in flight on its mbarrier: once a wait has given up, the
        // stage's previous fill may still be landing
        if (!waits_ok && ((filled >> s) & 1u)) drain_stage(s);
        filled |= 1u << s;
        odd ^= 1u << s;
        float *st = stages + s * L::STAGE_FLOATS;
        const unsigned bar = su32(&full[s]);
        st_mbar_expect(bar, L::TX_BYTES);
        const int x = i0 - SHX + sp.hx, y = j0, z = q + 1;  // the allocation starts at (-hx, -1, -1)
#pragma unroll
        for (int f = 0; f < 9; ++f) st_tma3(su32(st + f * SBOX), &sp.maps.st[f], x, y, z, bar);
#pragma unroll
        for (int f = 0; f < L::NC + L::NW; ++f) st_tma3(su32(st + (9 + f) * SBOX), &sp.maps.mt[f], x, y, z, bar);
#pragma unroll
        for (int f = 0; f < L::NB; ++f) st_tma3(su32(st + L::NBIG * SBOX + f * SOWN), &sp.maps.bu[f], i0 + sp.hx, j0 + 1, q, bar);
    };
    if (tid == 0) {
        for (int s = 0; s < SNSTAGE; ++s) st_mbar_init(su32(&full[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(ps);
        issue(ps + 1);
        int n = 0;
        for (int e = 0; e < fa.nsrc && n < MAXSRC; ++e) {
            const SrcEntry q = fa.src[e];
            if (q.i >= i0 - 1 && q.i <= i0 + SX && q.j >= j0 - 1 && q.j <= j0 + SY && q.k >= ps && q.k <= k1) s_src[n++] = q;
        }
        *s_nsrc = n;
    }
    const int it = *fa.it_ptr;
    const T sval = (fa.nsrc > 0 && it >= 0 && it < fa.nstf) ? (T)fa.stf[it] : T(0);

    // recomputed ring: warps 0-1 syy on row j0-1, 2-3 sxy and 4-5 syz on row j0+SY (64 columns),
    // 6 sxx on column i0-1, 7 sxy and 8 sxz on column i0+SX (8 rows); one component per warp
    int hcomp = -1, hi = 0, hj = 0, hb = 0;
    if (warp < 6) {
        const int hl = ((warp & 1) << 5) + lane;
        hcomp = warp < 2 ? 4 : (warp < 4 ? 6 : 8);
        hi = i0 + hl;
        hj = warp < 2 ? j0 - 1 : j0 + SY;
        hb = (warp < 2 ? 0 : SY + 1) * SBW + hl + SHX;
    } else if (warp < 9 && lane < SY) {
        hcomp = warp == 6 ? 3 : (warp == 7 ? 6 : 7);
        hi = warp == 6 ? i0 - 1 : i0 + SX;
        hj = j0 + lane;
        hb = (lane + 1) * SBW + (warp == 6 ? SHX - 1 : SHX + SX);
    }
    const bool hin = hcomp >= 0 && hi >= -1 && hi <= nx && hj >= -1 && hj <= ny;
    const HaloConst<T> hcst = hin ? halo_const<T, MODEL, DAMP>(a, hcomp, hi, hj) : HaloConst<T>{T(0), T(0), T(0), T(0)};
    // comp 7 / 8 difference Vx / Vy across planes: the value at the ring position on plane p-1
    T hvm = T(0);
    const bool hvm_on = hin && (hcomp == 7 || hcomp == 8) && hi >= 0 && hi < nx && hj >= 0 && hj < ny;
    if (hvm_on) hvm = ld(a.f[hcomp == 7 ? 0 : 1] + (long long)hi + (long long)hj * sx + (long long)(ps - 1) * sy);

    // column damping
    T wavx = T(0), wavy = T(0), wxi = T(0), wyj = T(0), pxy = T(0), wxm = T(0), wym = T(0);
    if (in_grid) {
        if (DAMP == DAMP_PML1D) {
            wxi = ld(a.w1[0] + i);
            wyj = ld(a.w1[1] + j);
            wavx = T(0.5) * (ld(a.w1[0] + i + 1) + wxi);
            wavy = T(0.5) * (ld(a.w1[1] + j + 1) + wyj);
            if (i > 0) wxm = ld(a.w1[0] + i - 1);
            if (j > 0) wym = ld(a.w1[1] + j - 1);
        } else if (DAMP == DAMP_SEP) {
            pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
        }
    }
    const bool do_x = in_grid && i >= 1 && j >= 1 && (j < ny - 1);
    const bool do_y = in_grid && i >= 1 && j >= 1 && (i < nx - 1);
    const bool do_z = in_grid && i >= 1 && j >= 1 && (i < nx - 1) && (j < ny - 1);
    const bool bxz = in_grid && i > 0 && row_bc;  // BC1 rewrites sxz(i, j, 1)
    const bool byz = in_grid && j > 0;            // BC1 rewrites syz(i, j, 1)

    long long c = (long long)i + (long long)j * sx + (long long)ps * sy;
    const int o = (ty + 1) * SBW + tx + SHX;  // the own cell in a staged box
    // own column, old state: V(p-1) and Vz(p-1) (the velocity update's old V, sigma's k-1 terms)
    T vx_m = T(0), vy_m = T(0), vz_km1 = T(0), wz_k = T(0);
    if (in_grid) {
        vx_m = ld(a.f[0] + c - sy);
        vy_m = ld(a.f[1] + c - sy);
        vz_km1 = ld(a.f[2] + c - sy);
        if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + ps);
    }
    T szz_m = T(0), szz_mm = T(0);  // szz(p-1), szz(p-2) of the own column
    T w_prev = T(0);                // the weight (3-D) or z profile (separable) of the last stress update
    __syncthreads();                // barriers initialised, sources listed
    const int nloc = *s_nsrc;

    for (int p = ps; p <= k1; ++p, c += sy) {
        const bool compute = (p < nz);
        const bool halo = (p >= max(1, k0)) && (p < k1);
        const bool write = (p >= k0) && (p < k1);
        const bool vplane = (p - 1 >= max(1, k0)) && (p - 1 < k1);
        const bool bc1p = (p == 2 && k0 == 0);  // BC1 rewrites plane 1 from this plane
        const int b = p % 3, pb = (p + 2) % 3;
        if (tid == 0 && p + 2 <= plast) issue(p + 2);  // the stage of plane p-1: free since the last barrier
        const float *Sp = stages + (p % SNSTAGE) * L::STAGE_FLOATS;
        const float *Sn = stages + ((p + 1) % SNSTAGE) * L::STAGE_FLOATS;
        bool got = st_mbar_wait(su32(&full[p % SNSTAGE]), (unsigned)((p - ps) / SNSTAGE) & 1u, wait_limit);
        got = st_mbar_wait(su32(&full[(p + 1) % SNSTAGE]), (unsigned)((p + 1 - ps) / SNSTAGE) & 1u, wait_limit) && got;
        waits_ok = waits_ok && got;

        T sv[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
        T xz1 = T(0), yz1 = T(0);
        // velocity side of plane p-1: old V and weights from registers, buoyancy from this stage
        const T v0 = vx_m, v1 = vy_m, v2 = vz_km1;
        T bxv = a.bx, byv = a.by, bzv = a.bz, wv = T(0);
        if (vplane && in_grid) {
            if (MODEL == MODEL_ORTHO) {
                const float *B = Sp + L::NBIG * SBOX + ty * SX + tx;
                bxv = B[0];
                byv = B[SOWN];
                bzv = B[2 * SOWN];
                wv = (DAMP == DAMP_W3D) ? w_prev : pxy * w_prev;
            } else {
                wv = ld(a.w1[2] + p - 2);
            }
        }
        const T wzp = (DAMP == DAMP_W3D) ? T(0) : ld(a.w1[2] + p);  // the z profile at plane p
        const T vz_k = Sp[2 * SBOX + o];

        if (compute) {
            if (in_grid) {
                StressIn<T, MODEL, DAMP> q;
                const float *Vx = Sp, *Vy = Sp + SBOX, *Vz = Sp + 2 * SBOX;
                q.vx = Vx[o];
                q.vx_ip = Vx[o + 1];
                q.vx_jm = Vx[o - SBW];
                q.vy = Vy[o];
                q.vy_jp = Vy[o + SBW];
                q.vy_im = Vy[o - 1];
                q.vz_p = Sn[2 * SBOX + o];
                q.vz_im = Vz[o - 1];
                q.vz_jm = Vz[o - SBW];
#pragma unroll
                for (int f = 0; f < 6; ++f) q.s[f] = Sp[(3 + f) * SBOX + o];
#pragma unroll
                for (int f = 0; f < L::NC; ++f) q.c[f] = Sp[(9 + f) * SBOX + o];
                if (MODEL == MODEL_ISO) q.w = ld(a.w1[2] + p + 1);
                else q.w = (DAMP == DAMP_W3D) ? Sp[(9 + L::NC) * SBOX + o] : wzp;
                const T Vxx = (q.vx_ip - q.vx) * rdx;
                const T Vyy = (q.vy_jp - q.vy) * rdy;
                const T Vzz = (q.vz_p - vz_k) * rdz;
                if (MODEL == MODEL_ISO) {
                    const T c11 = q.c[0], c12 = q.c[1];
                    sv[0] = nrm_iso(wavx, q.s[0], dt, c11, c12, c12, Vxx, Vyy, Vzz);
                    sv[1] = nrm_iso(wavy, q.s[1], dt, c12, c11, c12, Vxx, Vyy, Vzz);
                    sv[2] = nrm_iso(T(0.5) * (q.w + wz_k), q.s[2], dt, c12, c12, c11, Vxx, Vyy, Vzz);
                    const T c66dt = a.c66 * dt;
                    sv[3] = shr_iso(wz_k * wyj * wxi, q.s[3], c66dt, q.vy - q.vy_im, rdx, q.vx - q.vx_jm, rdy);
                    sv[4] = shr_iso(wyj * wz_k * wxi, q.s[4], c66dt, vz_k - q.vz_im, rdx, q.vx - vx_m, rdz);
                    sv[5] = shr_iso(wxi * wyj * wz_k, q.s[5], c66dt, q.vy - vy_m, rdz, vz_k - q.vz_jm, rdy);
                    wz_k = q.w;
                } else {
                    const T W = (DAMP == DAMP_W3D) ? q.w : pxy * q.w;
                    w_prev = q.w;
                    sv[0] = nrm_ortho(q.s[0], W, dt, q.c[0], q.c[3], q.c[4], Vxx, Vyy, Vzz);
                    sv[1] = nrm_ortho(q.s[1], W, dt, q.c[3], q.c[1], q.c[5], Vxx, Vyy, Vzz);
                    sv[2] = nrm_ortho(q.s[2], W, dt, q.c[4], q.c[5], q.c[2], Vxx, Vyy, Vzz);
                    const T xy = shr_ortho(q.s[3], W, dt, q.c[6], q.vy - q.vy_im, a.dx, a.rdx, q.vx - q.vx_jm, a.dy, a.rdy,
                                           a.fdiv != 0);
                    const T xz = shr_ortho(q.s[4], W, dt, q.c[7], vz_k - q.vz_im, a.dx, a.rdx, q.vx - vx_m, a.dz, a.rdz,
                                           a.fdiv != 0);
                    const T yz = shr_ortho(q.s[5], W, dt, q.c[8], q.vy - vy_m, a.dz, a.rdz, vz_k - q.vz_jm, a.dy, a.rdy,
                                           a.fdiv != 0);
                    sv[3] = (i > 0 && j > 0) ? xy : q.s[3];
                    sv[4] = (i > 0 && p > 0) ? xz : q.s[4];
                    sv[5] = (j > 0 && p > 0) ? yz : q.s[5];
                }
                if (p == 0 && row_bc) sv[2] = T(0);  // BC1 szz (OK4:279)
                vx_m = q.vx;
                vy_m = q.vy;
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = s_src[e];
                    if (q2.k == p && q2.i == i && q2.j == j && inject_when(a, q2, fa.order) == 1)
                        sv[q2.comp - 3] = sv[q2.comp - 3] + (T)q2.coef * sval;
                }
            }
            // this warp's recomputed ring position
            T h = T(0), h1 = T(0);
            if (halo && hin) {
                h = staged_sigma<MODEL, DAMP>(a, hcomp, hi, hj, p, hb, Sp, Sn, hvm, hcst, wzp);
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = s_src[e];
                    if (q2.k == p && q2.i == hi && q2.j == hj && q2.comp == hcomp && inject_when(a, q2, fa.order) == 1)
                        h = h + (T)q2.coef * sval;
                }
            }
            // BC1 (OK4:281-282): sxz / syz on plane 1 from plane 2, then the injections that come after it
            if (bc1p) {
                xz1 = a.third * sv[4];
                yz1 = a.third * sv[5];
                const bool hbc = (hcomp == 7 || hcomp == 8) && hin && bc1_plane1(a, hcomp, hi, hj);
                if (hbc) h1 = a.third * h;
                for (int e = 0; e < nloc; ++e) {
                    const SrcEntry q2 = s_src[e];
                    if (inject_when(a, q2, fa.order) != 2) continue;
                    const T add = (T)q2.coef * sval;
                    if (in_grid && q2.i == i && q2.j == j) {
                        if (q2.k == 1) {
                            if (q2.comp == 7) xz1 = xz1 + add;
                            else yz1 = yz1 + add;
                        } else {
                            sv[q2.comp - 3] = sv[q2.comp - 3] + add;
                        }
                    } else if (hbc && q2.i == hi && q2.j == hj && q2.comp == hcomp) {
                        if (q2.k == 1) h1 = h1 + add;
                        else h = h + add;
                    }
                }
            }
            if (halo) {
                StagedStress &S = stg(b);
                S.xx[ty][tx + 1] = sv[0];
                S.yy[ty + 1][tx] = sv[1];
                S.xy[ty][tx] = sv[3];
                S.xz[ty][tx] = sv[4];
                S.yz[ty][tx] = sv[5];
                if (hcomp >= 0) {
                    if (warp < 2) S.yy[0][hb - SHX] = h;
                    else if (warp < 4) S.xy[SY][hb - (SY + 1) * SBW - SHX] = h;
                    else if (warp < 6) S.yz[SY][hb - (SY + 1) * SBW - SHX] = h;
                    else if (warp == 6) S.xx[lane][0] = h;
                    else if (warp == 7) S.xy[lane][SX] = h;
                    else S.xz[lane][SX] = h;
                }
                if (bc1p) {  // plane 1 is buffer 1
                    StagedStress &S1 = stg(1);
                    if (bxz) S1.xz[ty][tx] = xz1;
                    if (byz) S1.yz[ty][tx] = yz1;
                    if ((hcomp == 7 || hcomp == 8) && hin && bc1_plane1(a, hcomp, hi, hj)) {
                        if (hcomp == 8) S1.yz[SY][hb - (SY + 1) * SBW - SHX] = h1;
                        else S1.xz[lane][SX] = h1;
                    }
                }
            }
            if (write && in_grid) {
#pragma unroll
                for (int f = 0; f < 6; ++f) fa.o[3 + f][c] = sv[f];
                if (bc1p) {
                    if (bxz) fa.o[7][c - sy] = xz1;
                    if (byz) fa.o[8][c - sy] = yz1;
                }
            }
        }
        if (hvm_on) hvm = Sp[(hcomp == 7 ? 0 : 1) * SBOX + hb];  // the ring position's Vx / Vy on plane p
        __syncthreads();  // plane p staged; every read of plane stage p done

        // velocity of plane p-1 (OK4:346-378 / ANISO:358-389)
        if (vplane && in_grid) {
            const StagedStress &S = stg(pb);
            const T sxz_p = sv[4], syz_p = sv[5];
            const T dSx = (S.xx[ty][tx + 1] - S.xx[ty][tx]) * rdx + (S.xy[ty + 1][tx] - S.xy[ty][tx]) * rdy +
                          (sxz_p - S.xz[ty][tx]) * rdz;
            const T dSy = (S.yy[ty + 1][tx] - S.yy[ty][tx]) * rdy + (S.xy[ty][tx + 1] - S.xy[ty][tx]) * rdx +
                          (syz_p - S.yz[ty][tx]) * rdz;
            const T dSz = (szz_m - szz_mm) * rdz + (S.xz[ty][tx + 1] - S.xz[ty][tx]) * rdx + (S.yz[ty + 1][tx] - S.yz[ty][tx]) * rdy;
            T ax, ay, az;
            if (MODEL == MODEL_ISO) { ax = wxm; ay = wym; az = wv; }
            else { ax = ay = az = wv; }
            T cp = T(0);
            const T nvx = vel_update<T, MODEL, false>(a, v0, dSx, ax, bxv, cp);
            const T nvy = vel_update<T, MODEL, false>(a, v1, dSy, ay, byv, cp);
            const T nvz = vel_update<T, MODEL, false>(a, v2, dSz, az, bzv, cp);
            const long long cv = c - sy;
            const int kv = p - 1;
            if (do_x && kv < nz - 1) fa.o[0][cv] = nvx;
            if (do_y && kv < nz - 1) fa.o[1][cv] = nvy;
            if (do_z) fa.o[2][cv] = nvz;
        }
        vz_km1 = vz_k;
        szz_mm = szz_m;
        szz_m = sv[2];
    }
    // A wait that gave up may leave copies in flight: before the CTA's shared memory goes away,
    // thread 0 waits (bounded) until every stage has completed one phase per fill it issued --
    // issued copies always land, so this ends as soon as they have.
    if (tid == 0 && (!waits_ok || *(volatile int *)&g_staged_err)) {
        for (int s = 0; s < SNSTAGE; ++s)
            if ((filled >> s) & 1u) drain_stage(s);
    }
}

}  // namespace ewf
