// ewfd_kernels.cuh -- sm_103a kernels of the staggered-grid elastic FDTD time step.
//
// Device layout ("box"): every field -- the 9 staggered state fields, the material fields and
// the 3-D damping field -- lives in one padded geometry shared by all of them:
//   element (i,j,k) at base[i + j*sx + k*sy],  i in [-HX, sx-HX), j in [-1, ny+2), k in [-1, nz+2)
// with HX = 128 B / sizeof(T) so that i = 0 starts a 128-byte line, sx a multiple of 32 and
// the base pointer placed at (0,0,0).  The reference's staggered extents (Vx is (nx+1,ny,nz),
// sxy is (nx+1,ny+1,nz) and so on) all fit inside; cells outside an array's own extent are
// zero and are never written, which makes every neighbour read of the reference stencil an
// in-bounds read of a zero (the reference reads a wrapped neighbour there, e.g. OK4:323-329,
// only for cells whose value is never read back).
//
// One time step (reference order OK4:485-505 / ANISO:519-555):
//   k_stress    stress update + damping, free surface BC1 fused at planes k = 0..2, point sources
//               applied by the threads that own their cells
//   k_inject    point injection for sources outside the stress kernel's cells (before-BC1
//               semantics replayed exactly), and for the other step forms
//   k_velocity  velocity update + damping (optionally Kahan-compensated)
//   k_record    receiver gather into FP64 traces; advances the device step counter
// Expression order follows the reference so that an FMA-free build is bit-identical to the
// reference's FMA-free build.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ewf {

enum { MODEL_ISO = 0, MODEL_ORTHO = 1, MODEL_ISOHET = 2 };
enum { DAMP_PML1D = 0, DAMP_W3D = 1, DAMP_SEP = 2, DAMP_PERCOMP = 3 };

// Tile of the z-marching kernels: one thread per (i,j) column, a CTA covers TX x TY columns
// and a chunk of planes.
constexpr int TX = 32;
constexpr int TY = 8;

template <typename T>
struct StepArgs {
    T *f[9];          // Vx Vy Vz sxx syy szz sxy sxz syz
    T *comp[3];       // Kahan compensation of Vx Vy Vz (null unless compensated)
    const T *m[12];   // iso: c11 c12 | ortho: C11 C22 C33 C12 C13 C23 C66xy C55xz C44yz Bx By Bz
    const T *w1[3];   // iso: PML profiles (n+1 each) | separable: per-axis factors (n each)
    const T *w3;      // 3-D damping field (box layout)
    const T *w6[6];   // per-component weights of Vx/sxx, Vy/syy, Vz/szz, sxy, sxz, syz (box layout)
    long long sy;     // plane pitch of materials / damping, elements
    int sx;           // row pitch of materials / damping, elements
    int R;            // right-hand sides interleaved along x in the state arrays (1: one source)
    int sxs;          // state row pitch (R * sx)
    long long sys;    // state plane pitch
    int nx, ny, nz;
    int bc1_rows;     // rows j < bc1_rows get the szz / sxz free-surface rule (OK4:279-281)
    int kchunk;       // planes per CTA
    T dt, rdt, dx, dy, dz, rdx, rdy, rdz;
    T c66, bx, by, bz;  // isotropic scalars (OK4:405-407)
    T c44, c55;         // per-component-weight scheme: shear moduli of yz and xz
    T third;            // (T)1/(T)3 of BC1
    int fdiv;           // 1: div_spacing may take the reciprocal path for dx, dy, dz (verified)
    T vdamp;            // linear velocity damping (16 km scheme), 0 = off
    int bc1;            // 1: BC1 after the stress update (stress_store, inject_entry); 0: none
    int smu_on;         // isotropic 1-D PML scheme: shear modulus smu instead of c66 on plane k = 1
    T smu;
    int l2pf;           // two-kernel step: the velocity kernel asks L2 for its inputs this many planes ahead (0: off)
};

struct SrcEntry {
    int comp, i, j, k;
    double coef;
};

// Point sources applied by the stress kernel itself (the two-kernel step): the thread that owns an
// entry's column applies it right after its stores of the entry's plane -- for sxz / syz on plane
// 1, after plane 2, whose update BC1 copies onto plane 1 -- with k_inject's arithmetic
// (inject_entry), so the result is bit-identical to the separate launch.  [i0, i1] x [j0, j1]
// bounds the entries' columns, so every other thread skips them with one test per plane.
struct StressSrc {
    const SrcEntry *src;  // nsrc entries, every one inside the stress kernel's cells (i < nx, j < ny, k < nz)
    int nsrc;             // 0: none (k_inject applies the sources, if any)
    const double *stf;
    int nstf;
    const int *it_ptr;
    int order;            // 0: before BC1 (OK4), 1: after (ANISO)
    int i0, i1, j0, j1;   // bounding box of the entries' columns
    int k1;               // last effective plane of any entry
};

// Receivers sampled by the velocity kernel itself (the two-kernel step): the thread that owns a
// receiver's column writes the trace sample right after its update of the receiver's plane, the
// value k_record would read (the new velocity where the update writes the cell, the old one where
// it does not).  col_first[j*nx + i] is the first entry of the column's receivers (-1: none),
// entries are (k, component, trace row, next entry of the column or -1).  The step counter is read
// at it_rd and, by one thread of the launch, written plus one at it_wr (a second location, so no
// thread of the launch can read the new value).  col_first null: k_record samples; it_wr null:
// k_record advances the counter.
struct RecFuse {
    const int *col_first;
    const int4 *ent;
    double *traces;
    int trace_len;
    const int *it_rd;
    int *it_wr;
};

// The plane after whose stores the stress kernel applies an entry.
__host__ __device__ __forceinline__ int fused_src_plane(int comp, int k) { return (k == 1 && (comp == 7 || comp == 8)) ? 2 : k; }

template <typename T>
__device__ __forceinline__ void inject_entry(const StepArgs<T> &a, const SrcEntry &q, T s, int order);

template <typename T>
__device__ __forceinline__ T ld(const T *p) { return __ldg(p); }

// Programmatic dependent launch.  The two-kernel step launches each kernel as a programmatic
// dependent of the previous one, so its CTAs are scheduled while the previous kernel's last wave
// runs instead of after a full launch gap.  Each kernel lets its dependent launch at once
// (pdl_trigger) and, before touching any state, waits until the previous grid has completed and
// its stores are visible (pdl_wait) -- so no read and no write moves ahead of the dependency.
// Launched without the attribute, both are no-ops.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// State loads.  COH = 0: the read-only path (the field is not written during the launch).
// COH = 1: a plain coherent load, for the wavefront step, where other CTAs of the same launch
// write the fields (ordered by its release/acquire flags).  COH = 2: a load cached in L2 only
// (ld.global.cg), for the sweep step's reads of values other CTAs wrote: no L1 line can hold
// an older copy.
template <int COH, typename T>
__device__ __forceinline__ T lds(const T *p)
{
    if constexpr (COH == 2) return __ldcg(p);
    else if constexpr (COH == 1) return *p;
    else return __ldg(p);
}

// ---------------------------------------------------------------------------------------------
// Division by a grid spacing.  The orthorhombic shear terms divide velocity differences by dx,
// dy, dz (ANISO:327-352), and six IEEE divisions per cell cost a sixth of the stress kernel's
// time.  div_spacing returns the same correctly rounded quotient through the reciprocal with
// Markstein's correction step (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Develop. 34(1), 1990): with r = RN(1/d),
// q = RN(x r), the residual e = x - q d is exact in one FMA, and RN(q + e r) is the quotient.
// For x = 0 or 2^-90 <= |x| <= 2^100 and 2^-10 <= d <= 2^30 every intermediate stays normal
// (the residual exact), so the result scales exactly with the binade of x; the library checks
// it against IEEE division over whole binades of x for each spacing on the device before it
// sets `ok` (ewfd.cu, fdiv_verified).  Other x, and unverified spacings, take IEEE division.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float div_spacing(float x, float d, float r, bool ok)
{
    const unsigned ax = __float_as_uint(x) & 0x7fffffffu;
    if (ok && (ax == 0u || ax - 0x12800000u <= 0x71800000u - 0x12800000u)) {  // 2^-90 .. 2^100
        const float q = __fmul_rn(x, r);
        const float e = __fmaf_rn(-q, d, x);
        return e == 0.f ? q : __fmaf_rn(e, r, q);  // e = 0: q is exact (and keeps the sign of -0)
    }
    return __fdiv_rn(x, d);
}
__device__ __forceinline__ double div_spacing(double x, double d, double, bool) { return x / d; }

// ---------------------------------------------------------------------------------------------
// Stress update.  Isotropic: OK4:285-331.  Orthorhombic: ANISO:287-356.  BC1: OK4:271-283.
//
// Each thread marches its (i,j) column over the CTA's planes.  All loads of a plane sit in one
// branch-free block (the box layout makes every neighbour read in-bounds) and the next plane's
// loads are issued before the current plane is computed, so ~25 independent loads per thread
// are always in flight; conditional updates become predicated stores.
// ---------------------------------------------------------------------------------------------
template <typename T, int MODEL, int DAMP>
struct StressIn {
    T vx, vx_ip, vx_jm;        // Vx(i,j,k), Vx(i+1), Vx(j-1)
    T vy, vy_jp, vy_im;        // Vy(i,j,k), Vy(j+1), Vy(i-1)
    T vz_p, vz_im, vz_jm;      // Vz(k+1), Vz(i-1,k), Vz(j-1,k)
    T s[6];                    // sxx syy szz sxy sxz syz at (i,j,k)
    T c[MODEL == MODEL_ISO ? 2 : (MODEL == MODEL_ISOHET ? 5 : 9)];
    T w;                       // iso: wz[k+1]; ortho, iso-het: W or pz[k]
    T pw[DAMP == DAMP_PERCOMP ? 6 : 1];  // per-component weights at the cell
};

// State part of a cell's stress inputs (c: state index, x stride R).
template <typename T, int MODEL, int DAMP, int RC, int COH = 0>
__device__ __forceinline__ void stress_load_state(const StepArgs<T> &a, long long c, StressIn<T, MODEL, DAMP> &q)
{
    const int R = RC ? RC : a.R;
    const int sx = (RC == 1) ? a.sx : a.sxs;
    const long long sy = (RC == 1) ? a.sy : a.sys;
    q.vx = lds<COH>(a.f[0] + c);
    q.vx_ip = lds<COH>(a.f[0] + c + R);
    q.vx_jm = lds<COH>(a.f[0] + c - sx);
    q.vy = lds<COH>(a.f[1] + c);
    q.vy_jp = lds<COH>(a.f[1] + c + sx);
    q.vy_im = lds<COH>(a.f[1] + c - R);
    q.vz_p = lds<COH>(a.f[2] + c + sy);
    q.vz_im = lds<COH>(a.f[2] + c - R);
    q.vz_jm = lds<COH>(a.f[2] + c - sx);
#pragma unroll
    for (int f = 0; f < 6; ++f) q.s[f] = a.f[3 + f][c];
}

// Material part (moduli, damping) of a cell's stress inputs (cm: material index, plane k).
template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ void stress_load_mat(const StepArgs<T> &a, long long cm, int k, StressIn<T, MODEL, DAMP> &q)
{
    if (MODEL == MODEL_ISO) {
        q.c[0] = ld(a.m[0] + cm);
        q.c[1] = ld(a.m[1] + cm);
        if (DAMP == DAMP_PERCOMP) {
#pragma unroll
            for (int f = 0; f < 6; ++f) q.pw[f] = ld(a.w6[f] + cm);
        } else {
            q.w = ld(a.w1[2] + k + 1);
        }
    } else if (MODEL == MODEL_ISOHET) {
        q.c[0] = ld(a.m[0] + cm);  // c11u_het
        q.c[1] = ld(a.m[3] + cm);  // c12u_het
#pragma unroll
        for (int f = 0; f < 3; ++f) q.c[2 + f] = ld(a.m[6 + f] + cm);  // c44u_het xy, xz, yz
        q.w = (DAMP == DAMP_W3D) ? ld(a.w3 + cm) : ld(a.w1[2] + k);
    } else {
#pragma unroll
        for (int f = 0; f < 9; ++f) q.c[f] = ld(a.m[f] + cm);
        q.w = (DAMP == DAMP_W3D) ? ld(a.w3 + cm) : ld(a.w1[2] + k);
    }
}
// c: state index (x stride R), cm: material index of the same cell
template <typename T, int MODEL, int DAMP, int RC, int COH = 0>
__device__ __forceinline__ void stress_load(const StepArgs<T> &a, long long c, long long cm, int k,
                                            StressIn<T, MODEL, DAMP> &q)
{
    stress_load_state<T, MODEL, DAMP, RC, COH>(a, c, q);
    stress_load_mat<T, MODEL, DAMP>(a, cm, k, q);
}

// damping factors constant along a column
template <typename T>
struct ColDamp {
    T wavx, wavy, wxi, wyj, pxy;
};
template <typename T, int DAMP>
__device__ __forceinline__ ColDamp<T> col_damp(const StepArgs<T> &a, int i, int j)
{
    ColDamp<T> d{T(0), T(0), T(0), T(0), T(0)};
    if (DAMP == DAMP_PML1D) {
        d.wxi = ld(a.w1[0] + i);
        d.wyj = ld(a.w1[1] + j);
        d.wavx = T(0.5) * (ld(a.w1[0] + i + 1) + d.wxi);
        d.wavy = T(0.5) * (ld(a.w1[1] + j + 1) + d.wyj);
    } else if (DAMP == DAMP_SEP) {
        d.pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
    }
    return d;
}

// The new stresses of cell (i, j, k): o = sxx syy szz sxy sxz syz; w_* = whether the shear
// component is written there.  vx_m, vy_m: Vx, Vy at k-1; vz_k: Vz at k; wz_k: wz[k] (iso).
template <typename T, int MODEL, int DAMP>
__device__ __forceinline__ void stress_math(const StepArgs<T> &a, const StressIn<T, MODEL, DAMP> &q,
                                            const ColDamp<T> &cd, int i, int j, int k, T vx_m, T vy_m, T vz_k,
                                            T wz_k, T (&o)[6], bool &w_xy, bool &w_xz, bool &w_yz)
{
    const T dt = a.dt, rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;
    const T Vxx = (q.vx_ip - q.vx) * rdx;
    const T Vyy = (q.vy_jp - q.vy) * rdy;
    const T Vzz = (q.vz_p - vz_k) * rdz;
    w_xy = true;
    w_xz = true;
    w_yz = true;
    if (MODEL == MODEL_ISO && DAMP == DAMP_PERCOMP) {
        const T c11 = q.c[0], c12 = q.c[1];
        // DC_Earthquake FastWaveED_GPU3D_v1.cu:313-315: each component's own 3-D weight
        o[0] = q.pw[0] * (q.s[0] + dt * (c11 * Vxx + c12 * Vyy + c12 * Vzz));
        o[1] = q.pw[1] * (q.s[1] + dt * (c12 * Vxx + c11 * Vyy + c12 * Vzz));
        o[2] = q.pw[2] * (q.s[2] + dt * (c12 * Vxx + c12 * Vyy + c11 * Vzz));
        // :318-320, the shear moduli c66 (xy), c55 (xz), c44 (yz); guarded like ANISO
        o[3] = q.pw[3] * (q.s[3] + a.c66 * dt * ((q.vy - q.vy_im) * rdx + (q.vx - q.vx_jm) * rdy));
        o[4] = q.pw[4] * (q.s[4] + a.c55 * dt * ((vz_k - q.vz_im) * rdx + (q.vx - vx_m) * rdz));
        o[5] = q.pw[5] * (q.s[5] + a.c44 * dt * ((q.vy - vy_m) * rdz + (vz_k - q.vz_jm) * rdy));
        w_xy = (i > 0 && j > 0);
        w_xz = (i > 0 && k > 0);
        w_yz = (j > 0 && k > 0);
    } else if (MODEL == MODEL_ISO) {
        const T c11 = q.c[0], c12 = q.c[1];
        // OK4:307-309
        o[0] = cd.wavx * (q.s[0] + dt * (c11 * Vxx + c12 * Vyy + c12 * Vzz));
        o[1] = cd.wavy * (q.s[1] + dt * (c12 * Vxx + c11 * Vyy + c12 * Vzz));
        o[2] = T(0.5) * (q.w + wz_k) * (q.s[2] + dt * (c12 * Vxx + c12 * Vyy + c11 * Vzz));
        // the diff_BC2_OK3 scheme's shear modulus on plane 1 (its FastWaveED_GPU3D_v1.cu:309-314)
        const T c66dt = ((a.smu_on && k == 1) ? a.smu : a.c66) * dt;
        // OK4:323, 326, 329 (no guards: zero-padded neighbours at the low edges)
        o[3] = wz_k * cd.wyj * cd.wxi * (q.s[3] + c66dt * ((q.vy - q.vy_im) * rdx + (q.vx - q.vx_jm) * rdy));
        o[4] = cd.wyj * wz_k * cd.wxi * (q.s[4] + c66dt * ((vz_k - q.vz_im) * rdx + (q.vx - vx_m) * rdz));
        o[5] = cd.wxi * cd.wyj * wz_k * (q.s[5] + c66dt * ((q.vy - vy_m) * rdz + (vz_k - q.vz_jm) * rdy));
    } else if (MODEL == MODEL_ISOHET) {
        const T W = (DAMP == DAMP_W3D) ? q.w : cd.pxy * q.w;
        const T c11 = q.c[0], c12 = q.c[1];
        // 9kmst.cu:316-318
        o[0] = q.s[0] * W + dt * (c11 * Vxx + c12 * Vyy + c12 * Vzz);
        o[1] = q.s[1] * W + dt * (c12 * Vxx + c11 * Vyy + c12 * Vzz);
        o[2] = q.s[2] * W + dt * (c12 * Vxx + c12 * Vyy + c11 * Vzz);
        // 9kmst.cu:321-325: edge shear moduli, derivatives times the reciprocal spacing
        o[3] = q.s[3] * W + q.c[2] * dt * ((q.vy - q.vy_im) * rdx + (q.vx - q.vx_jm) * rdy);
        o[4] = q.s[4] * W + q.c[3] * dt * ((vz_k - q.vz_im) * rdx + (q.vx - vx_m) * rdz);
        o[5] = q.s[5] * W + q.c[4] * dt * ((q.vy - vy_m) * rdz + (vz_k - q.vz_jm) * rdy);
        w_xy = (i > 0 && j > 0);
        w_xz = (i > 0 && k > 0);
        w_yz = (j > 0 && k > 0);
    } else {
        const T W = (DAMP == DAMP_W3D) ? q.w : cd.pxy * q.w;
        // ANISO:312-325 (c[]: C11 C22 C33 C12 C13 C23 C66 C55 C44)
        o[0] = q.s[0] * W + dt * (q.c[0] * Vxx + q.c[3] * Vyy + q.c[4] * Vzz);
        o[1] = q.s[1] * W + dt * (q.c[3] * Vxx + q.c[1] * Vyy + q.c[5] * Vzz);
        o[2] = q.s[2] * W + dt * (q.c[4] * Vxx + q.c[5] * Vyy + q.c[2] * Vzz);
        // ANISO:327-352 (shear derivatives divide by the spacing)
        const bool fd = a.fdiv != 0;
        const T dVx_dy = div_spacing(q.vx - q.vx_jm, a.dy, a.rdy, fd);
        const T dVy_dx = div_spacing(q.vy - q.vy_im, a.dx, a.rdx, fd);
        o[3] = q.s[3] * W + dt * q.c[6] * (dVy_dx + dVx_dy);
        const T dVx_dz = div_spacing(q.vx - vx_m, a.dz, a.rdz, fd);
        const T dVz_dx = div_spacing(vz_k - q.vz_im, a.dx, a.rdx, fd);
        o[4] = q.s[4] * W + dt * q.c[7] * (dVz_dx + dVx_dz);
        const T dVy_dz = div_spacing(q.vy - vy_m, a.dz, a.rdz, fd);
        const T dVz_dy = div_spacing(vz_k - q.vz_jm, a.dy, a.rdy, fd);
        o[5] = q.s[5] * W + dt * q.c[8] * (dVy_dz + dVz_dy);
        w_xy = (i > 0 && j > 0);
        w_xz = (i > 0 && k > 0);
        w_yz = (j > 0 && k > 0);
    }
}

// Stores the new stresses of cell c (plane k; sys: state plane pitch), with BC1 (when a.bc1):
// szz = 0 on plane 0 and, from the freshly updated plane 2, sxz / syz on plane 1 (OK4:279-282).
template <typename T>
__device__ __forceinline__ void stress_store(const StepArgs<T> &a, long long c, long long sys, int k, int i, int j,
                                             bool row_bc, const T (&o)[6], bool w_xy, bool w_xz, bool w_yz)
{
    a.f[3][c] = o[0];
    a.f[4][c] = o[1];
    a.f[5][c] = (k == 0 && row_bc && a.bc1) ? T(0) : o[2];
    if (w_xy) a.f[6][c] = o[3];
    if (w_xz) a.f[7][c] = o[4];
    if (w_yz) a.f[8][c] = o[5];
    if (k == 2 && a.bc1) {
        if (i > 0 && row_bc) a.f[7][c - sys] = a.third * o[4];
        if (j > 0) a.f[8][c - sys] = a.third * o[5];
    }
}

// L2 prefetch of one 128-byte line (a hint: no completion to wait for, no register written).
__device__ __forceinline__ void l2_prefetch_line(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The column (X = i*R + r, j) over planes [k0, k1): X runs over the cells of every RHS.
// RC: R known at compile time (1: one RHS, state and materials share one index; 0: a.R).
// SOFF (with RC = 1): the state lives soff elements after the materials' index (one of several
// right-hand sides in separate boxes of the same geometry).  COH: coherent state loads (lds).
template <typename T, int MODEL, int DAMP, int RC, bool SOFF = false, int COH = 0, bool SRC = false>
__device__ __forceinline__ void stress_column(const StepArgs<T> &a, int X, int j, int k0, int k1, long long soff = 0,
                                              const StressSrc &ss = StressSrc{})
{
    constexpr bool SEP = (RC != 1) || SOFF;  // separate state and material indices
    const int R = RC ? RC : a.R;
    const int i = (RC == 1) ? X : X / R;
    if (i >= a.nx || j >= a.ny) return;
    const int sxs = (RC == 1) ? a.sx : a.sxs;
    const long long sys = (RC == 1) ? a.sy : a.sys, sy = a.sy;
    const ColDamp<T> cd = col_damp<T, DAMP>(a, i, j);
    const bool row_bc = (j < a.bc1_rows);

    long long c = (long long)X + (long long)j * sxs + (long long)k0 * sys + (SOFF ? soff : 0);
    long long cm = !SEP ? c : (RC == 1) ? c - soff : (long long)i + (long long)j * a.sx + (long long)k0 * sy;
    T vx_m = lds<COH>(a.f[0] + c - sys);  // Vx(k-1)
    T vy_m = lds<COH>(a.f[1] + c - sys);  // Vy(k-1)
    T vz_k = lds<COH>(a.f[2] + c);        // Vz(k)
    T wz_k = T(0);
    if (DAMP == DAMP_PML1D) wz_k = ld(a.w1[2] + k0);
    StressIn<T, MODEL, DAMP> nxt;
    stress_load<T, MODEL, DAMP, RC, COH>(a, c, SEP ? cm : c, k0, nxt);
    // point sources on this column (SRC: the two-kernel step's stress kernel)
    bool src_col = false;
    T s_src = T(0);
    if (SRC && ss.nsrc > 0 && i >= ss.i0 && i <= ss.i1 && j >= ss.j0 && j <= ss.j1 && k0 <= ss.k1) {
        const int it = *ss.it_ptr;
        src_col = it >= 0 && it < ss.nstf;  // the host validates the step range; never read past Src
        if (src_col) s_src = (T)ss.stf[it];
    }

    for (int k = k0; k < k1; ++k, c += sys) {
        if (SEP && k > k0) cm += sy;
        const StressIn<T, MODEL, DAMP> q = nxt;
        if (k + 1 < k1) stress_load<T, MODEL, DAMP, RC, COH>(a, c + sys, SEP ? cm + sy : c + sys, k + 1, nxt);
        T o[6];
        bool w_xy, w_xz, w_yz;
        stress_math<T, MODEL, DAMP>(a, q, cd, i, j, k, vx_m, vy_m, vz_k, wz_k, o, w_xy, w_xz, w_yz);
        stress_store<T>(a, c, sys, k, i, j, row_bc, o, w_xy, w_xz, w_yz);
        if (SRC && src_col && k <= ss.k1) {
            for (int e = 0; e < ss.nsrc; ++e) {
                const SrcEntry q_e = ss.src[e];
                if (q_e.i == i && q_e.j == j && fused_src_plane(q_e.comp, q_e.k) == k) inject_entry(a, q_e, s_src, ss.order);
            }
        }
        if (MODEL == MODEL_ISO && DAMP == DAMP_PML1D) wz_k = q.w;
        vx_m = q.vx;
        vy_m = q.vy;
        vz_k = q.vz_p;
    }
}

// The two-kernel step's CTAs are TX x blockDim.y columns: blockDim.y (the tile height, chosen by
// the autotuner) is at most SPLIT_MAX_TY for FP32 and TY for FP64.  The bounds keep the
// register budget of 4 CTAs of 32 x 8 columns per SM in FP32 (64 per thread) for every height.
constexpr int SPLIT_MAX_TY = 16;
template <typename T>
constexpr int split_max_threads() { return sizeof(T) == 4 ? TX * SPLIT_MAX_TY : TX * TY; }
template <typename T>
constexpr int split_min_ctas() { return sizeof(T) == 4 ? 2 : 1; }

template <typename T, int MODEL, int DAMP>
__global__ void __launch_bounds__(split_max_threads<T>(), split_min_ctas<T>()) k_stress(const StepArgs<T> a,
                                                                                        const StressSrc ss)
{
    pdl_trigger();
    pdl_wait();
    const int k0 = blockIdx.z * a.kchunk;
    stress_column<T, MODEL, DAMP, 1, false, 0, true>(a, blockIdx.x * TX + threadIdx.x,
                                                     blockIdx.y * blockDim.y + threadIdx.y, k0,
                                                     min(k0 + a.kchunk, a.nz), 0, ss);
}

// ---------------------------------------------------------------------------------------------
// Point injection sigma_c += coef * Src[it], one thread, entries in order.
// order 0 replays "inject, then BC1" (OK4:336-342 run inside the stress kernel, BC1 after it):
// an entry on a cell that BC1 overwrites is dropped, and an entry on the plane BC1 copies from
// refreshes the copy.  order 1 is "BC1, then inject" (ANISO:533-535).
// ---------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void inject_entry(const StepArgs<T> &a, const SrcEntry &q, T s, int order)
{
    const long long c = (long long)q.i * a.R + (long long)q.j * a.sxs + (long long)q.k * a.sys;
    T *f = a.f[q.comp];
    if (order == 0) {
        const bool row_bc = a.bc1 && q.j < a.bc1_rows;
        const bool xz_bc = (q.comp == 7) && q.i > 0 && q.i < a.nx && row_bc;
        const bool yz_bc = a.bc1 && (q.comp == 8) && q.j > 0 && q.j < a.ny && q.i < a.nx;
        if ((q.comp == 5 && q.k == 0 && row_bc) || ((xz_bc || yz_bc) && q.k == 1)) return;
        f[c] = f[c] + (T)q.coef * s;
        if ((xz_bc || yz_bc) && q.k == 2) f[c - a.sys] = a.third * f[c];
    } else {
        f[c] = f[c] + (T)q.coef * s;
    }
}

template <typename T>
__global__ void k_inject(const StepArgs<T> a, const SrcEntry *__restrict__ src, int nsrc,
                         const double *__restrict__ stf, int nstf, const int *__restrict__ it_ptr, int order)
{
    pdl_trigger();
    pdl_wait();
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int it = *it_ptr;
    if (it < 0 || it >= nstf) return;  // the host validates the step range; never read past Src
    const T s = (T)stf[it];
    for (int e = 0; e < nsrc; ++e) inject_entry(a, src[e], s, order);
}

// ---------------------------------------------------------------------------------------------
// Velocity update.  Isotropic: OK4:346-378.  Orthorhombic: ANISO:358-389.
// KAHAN: V = a*V + inc with the rounding error carried in comp[] (compensated summation).
// Same structure as k_stress: hoisted, prefetched loads; predicated stores.
// ---------------------------------------------------------------------------------------------
template <typename T, int MODEL, int DAMP, bool KAHAN>
struct VelIn {
    T sxx, sxx_im, syy, syy_jm, szz;
    T sxy, sxy_jp, sxy_ip;
    T sxz_p, sxz_ip, syz_p, syz_jp;   // sxz(k+1), sxz(i+1,k), syz(k+1), syz(j+1,k)
    T v[3];
    T b[MODEL == MODEL_ISO ? 1 : 3];
    T w;                              // iso: wz[k-1]; ortho: W or pz[k]
    T pw[DAMP == DAMP_PERCOMP ? 3 : 1];  // per-component weights of Vx, Vy, Vz
    T cp[KAHAN ? 3 : 1];
};

// The stresses around a cell that its velocity update reads (c: state index, x stride R).
template <typename T, int MODEL, int DAMP, bool KAHAN, int RC, int COH = 0>
__device__ __forceinline__ void vel_load_sigma(const StepArgs<T> &a, long long c, VelIn<T, MODEL, DAMP, KAHAN> &q)
{
    const int R = RC ? RC : a.R;
    const int sx = (RC == 1) ? a.sx : a.sxs;
    const long long sy = (RC == 1) ? a.sy : a.sys;
    q.sxx = lds<COH>(a.f[3] + c);
    q.sxx_im = lds<COH>(a.f[3] + c - R);
    q.syy = lds<COH>(a.f[4] + c);
    q.syy_jm = lds<COH>(a.f[4] + c - sx);
    q.szz = lds<COH>(a.f[5] + c);
    q.sxy = lds<COH>(a.f[6] + c);
    q.sxy_jp = lds<COH>(a.f[6] + c + sx);
    q.sxy_ip = lds<COH>(a.f[6] + c + R);
    q.sxz_p = lds<COH>(a.f[7] + c + sy);
    q.sxz_ip = lds<COH>(a.f[7] + c + R);
    q.syz_p = lds<COH>(a.f[8] + c + sy);
    q.syz_jp = lds<COH>(a.f[8] + c + sx);
}

// State part of a cell's velocity inputs: the stresses around the cell and the old velocities.
template <typename T, int MODEL, int DAMP, bool KAHAN, int RC, int COH = 0>
__device__ __forceinline__ void vel_load_state(const StepArgs<T> &a, long long c, VelIn<T, MODEL, DAMP, KAHAN> &q)
{
    vel_load_sigma<T, MODEL, DAMP, KAHAN, RC, COH>(a, c, q);
#pragma unroll
    for (int f = 0; f < 3; ++f) q.v[f] = a.f[f][c];
}

// Material part (buoyancy, damping) of a cell's velocity inputs (cm: material index, plane k).
template <typename T, int MODEL, int DAMP, bool KAHAN>
__device__ __forceinline__ void vel_load_mat(const StepArgs<T> &a, long long cm, int k, VelIn<T, MODEL, DAMP, KAHAN> &q)
{
    if (MODEL == MODEL_ISO && DAMP == DAMP_PERCOMP) {
#pragma unroll
        for (int f = 0; f < 3; ++f) q.pw[f] = ld(a.w6[f] + cm);
    } else if (MODEL == MODEL_ISO) {
        q.w = ld(a.w1[2] + k - 1);
    } else {
#pragma unroll
        for (int f = 0; f < 3; ++f) q.b[f] = ld(a.m[9 + f] + cm);
        q.w = (DAMP == DAMP_W3D) ? ld(a.w3 + cm) : ld(a.w1[2] + k);
    }
}
template <typename T, int MODEL, int DAMP, bool KAHAN, int RC, int COH = 0>
__device__ __forceinline__ void vel_load(const StepArgs<T> &a, long long c, long long cm, int k,
                                         VelIn<T, MODEL, DAMP, KAHAN> &q)
{
    vel_load_state<T, MODEL, DAMP, KAHAN, RC, COH>(a, c, q);
    vel_load_mat<T, MODEL, DAMP, KAHAN>(a, cm, k, q);
    if (KAHAN) {
#pragma unroll
        for (int f = 0; f < 3; ++f) q.cp[f] = a.comp[f][c];
    }
}

template <typename T, int MODEL, bool KAHAN>
__device__ __forceinline__ T vel_update(const StepArgs<T> &a, T V, T dS, T w_or_W, T b, T &cp)
{
    if (!KAHAN) {
        if (MODEL == MODEL_ISO) return w_or_W * (V * a.rdt + b * dS) * a.dt;
        const T r = (V * a.rdt * w_or_W + b * dS) * a.dt;
        return a.vdamp != T(0) ? r - a.vdamp * V : r;  // 16kmst.cu:337-349
    }
    const T aa = w_or_W;
    const T inc = (MODEL == MODEL_ISO) ? aa * (b * dS) * a.dt : b * dS * a.dt;
    const T y = inc - aa * cp;
    const T av = aa * V;
    const T t = av + y;
    cp = (t - av) - y;
    return t;
}

// damping factors constant along a velocity column
template <typename T>
struct VelDamp {
    T wxm, wym, pxy;
};
template <typename T, int DAMP>
__device__ __forceinline__ VelDamp<T> vel_damp(const StepArgs<T> &a, int i, int j)
{
    VelDamp<T> d{T(0), T(0), T(0)};
    if (DAMP == DAMP_PML1D) {
        d.wxm = ld(a.w1[0] + i - 1);
        d.wym = ld(a.w1[1] + j - 1);
    } else if (DAMP == DAMP_SEP) {
        d.pxy = ld(a.w1[0] + i) * ld(a.w1[1] + j);
    }
    return d;
}

// The new velocities of one cell: v = Vx Vy Vz (cp: Kahan compensations, updated in place).
// szz_m: szz at k-1; sxz_k, syz_k: sxz, syz at k.
template <typename T, int MODEL, int DAMP, bool KAHAN>
__device__ __forceinline__ void vel_math(const StepArgs<T> &a, const VelIn<T, MODEL, DAMP, KAHAN> &q,
                                         const VelDamp<T> &vd, T szz_m, T sxz_k, T syz_k, T (&v)[3], T (&cp)[3])
{
    const T rdx = a.rdx, rdy = a.rdy, rdz = a.rdz;
    const T dSx = (q.sxx - q.sxx_im) * rdx + (q.sxy_jp - q.sxy) * rdy + (q.sxz_p - sxz_k) * rdz;
    const T dSy = (q.syy - q.syy_jm) * rdy + (q.sxy_ip - q.sxy) * rdx + (q.syz_p - syz_k) * rdz;
    const T dSz = (q.szz - szz_m) * rdz + (q.sxz_ip - sxz_k) * rdx + (q.syz_jp - syz_k) * rdy;
    T ax, ay, az, bx, by, bz;
    if (MODEL == MODEL_ISO && DAMP == DAMP_PERCOMP) {
        // DC_Earthquake FastWaveED_GPU3D_v1.cu:344-360: each component's own 3-D weight
        ax = q.pw[0]; ay = q.pw[1]; az = q.pw[2];
        bx = a.bx; by = a.by; bz = a.bz;
    } else if (MODEL == MODEL_ISO) {
        ax = vd.wxm; ay = vd.wym; az = q.w;
        bx = a.bx; by = a.by; bz = a.bz;
    } else {
        const T W = (DAMP == DAMP_W3D) ? q.w : vd.pxy * q.w;
        ax = ay = az = W;
        bx = q.b[0]; by = q.b[1]; bz = q.b[2];
    }
    v[0] = vel_update<T, MODEL, KAHAN>(a, q.v[0], dSx, ax, bx, cp[0]);
    v[1] = vel_update<T, MODEL, KAHAN>(a, q.v[1], dSy, ay, by, cp[1]);
    v[2] = vel_update<T, MODEL, KAHAN>(a, q.v[2], dSz, az, bz, cp[2]);
}

// Stores the new velocities of cell c on plane k, within the ranges OK4:358, 365, 372.
template <typename T, bool KAHAN>
__device__ __forceinline__ void vel_store(const StepArgs<T> &a, long long c, int k, int i, int j, const T (&v)[3],
                                          const T (&cp)[3])
{
    if (j < a.ny - 1 && k < a.nz - 1) {
        a.f[0][c] = v[0];
        if (KAHAN) a.comp[0][c] = cp[0];
    }
    if (i < a.nx - 1 && k < a.nz - 1) {
        a.f[1][c] = v[1];
        if (KAHAN) a.comp[1][c] = cp[1];
    }
    if (i < a.nx - 1 && j < a.ny - 1) {
        a.f[2][c] = v[2];
        if (KAHAN) a.comp[2][c] = cp[2];
    }
}

// L2 prefetch of plane-ahead inputs of the velocity update for one warp's row of 32 cells: lane l
// asks for the 128-byte line of input field l (sxx..syz, Vx..Vz, then buoyancy, 3-D weights and
// compensation where the scheme reads them) that holds the row's cells.  This returns lane l's
// field (null: none); the row's line of plane k is at field + (c - lane) + k * plane pitch, c
// being the lane's element (the x pitch and the row start are 32-aligned).  (The stress kernel,
// already at the copy bandwidth, has no registers to spare for it.)  STATE_ONLY: the state fields
// alone (a right-hand side in a box of its own, soff elements after the materials' index: c is
// the state's index, and the shared material lines come from L2 for all right-hand sides).
template <typename T, int MODEL, int DAMP, bool KAHAN, bool STATE_ONLY = false>
__device__ __forceinline__ const T *vel_prefetch_field(const StepArgs<T> &a, int lane)
{
    if (lane < 6) return a.f[3 + lane];
    if (lane < 9) return a.f[lane - 6];
    if (STATE_ONLY) return nullptr;
    if (MODEL != MODEL_ISO && lane < 12) return a.m[lane];
    if (MODEL != MODEL_ISO && DAMP == DAMP_W3D && lane == 12) return a.w3;
    if (MODEL == MODEL_ISO && DAMP == DAMP_PERCOMP && lane >= 9 && lane < 12) return a.w6[lane - 9];
    if (KAHAN && lane >= 13 && lane < 16) return a.comp[lane - 13];
    return nullptr;
}

template <typename T, int MODEL, int DAMP, bool KAHAN, int RC, bool SOFF = false, int COH = 0, bool REC = false>
__device__ __forceinline__ void velocity_column(const StepArgs<T> &a, int X, int j, int kc0, int kc1, long long soff = 0,
                                                const RecFuse &rf = RecFuse{})
{
    constexpr bool SEP = (RC != 1) || SOFF;  // separate state and material indices (see stress_column)
    const int R = RC ? RC : a.R;
    const int i = (RC == 1) ? X : X / R;
    if (i < 1 || j < 1 || i >= a.nx || j >= a.ny) return;
    const int k0 = max(1, kc0);
    const int k1 = kc1;
    if (k0 >= k1) return;
    const int sxs = (RC == 1) ? a.sx : a.sxs;
    const long long sys = (RC == 1) ? a.sy : a.sys, sy = a.sy;
    const VelDamp<T> vd = vel_damp<T, DAMP>(a, i, j);

    long long c = (long long)X + (long long)j * sxs + (long long)k0 * sys + (SOFF ? soff : 0);
    long long cm = !SEP ? c : (RC == 1) ? c - soff : (long long)i + (long long)j * a.sx + (long long)k0 * sy;
    T szz_m = lds<COH>(a.f[5] + c - sys);
    T sxz_k = lds<COH>(a.f[7] + c);
    T syz_k = lds<COH>(a.f[8] + c);
    VelIn<T, MODEL, DAMP, KAHAN> nxt;
    vel_load<T, MODEL, DAMP, KAHAN, RC, COH>(a, c, SEP ? cm : c, k0, nxt);
    // the L2 prefetch's field for this lane (REC: the two-kernel step's velocity kernel)
    const T *pf_row = nullptr;
    if (REC && a.l2pf > 0) {
        pf_row = vel_prefetch_field<T, MODEL, DAMP, KAHAN, SOFF>(a, (int)threadIdx.x);
        if (pf_row) pf_row += c - (long long)threadIdx.x + (long long)a.l2pf * sys;
    }
    // receivers on this column (REC: the two-kernel step's velocity kernel)
    int r_first = -1, r_it = 0;
    if (REC && rf.col_first) {
        r_first = rf.col_first[(long long)j * a.nx + i];
        if (r_first >= 0) r_it = *rf.it_rd;
    }

    for (int k = k0; k < k1; ++k, c += sys) {
        if (SEP && k > k0) cm += sy;
        VelIn<T, MODEL, DAMP, KAHAN> q = nxt;
        if (k + 1 < k1) vel_load<T, MODEL, DAMP, KAHAN, RC, COH>(a, c + sys, SEP ? cm + sy : c + sys, k + 1, nxt);
        if (REC && pf_row && k + a.l2pf < k1) l2_prefetch_line(pf_row + (long long)(k - k0) * sys);
        T v[3], cp[3] = {KAHAN ? q.cp[0] : T(0), KAHAN ? q.cp[1] : T(0), KAHAN ? q.cp[2] : T(0)};
        vel_math<T, MODEL, DAMP, KAHAN>(a, q, vd, szz_m, sxz_k, syz_k, v, cp);
        vel_store<T, KAHAN>(a, c, k, i, j, v, cp);
        if (REC && r_first >= 0 && r_it >= 0 && r_it < rf.trace_len) {
            for (int e = r_first; e >= 0;) {
                const int4 re = rf.ent[e];
                if (re.x == k) {
                    // the cell's value after the update: vel_store's ranges decide new or old
                    const bool upd = re.y == 0 ? (j < a.ny - 1 && k < a.nz - 1)
                                   : re.y == 1 ? (i < a.nx - 1 && k < a.nz - 1) : (i < a.nx - 1 && j < a.ny - 1);
                    const T val = re.y == 0 ? (upd ? v[0] : q.v[0]) : re.y == 1 ? (upd ? v[1] : q.v[1]) : (upd ? v[2] : q.v[2]);
                    rf.traces[(long long)re.z * rf.trace_len + r_it] = (double)val;
                }
                e = re.w;
            }
        }
        szz_m = q.szz;
        sxz_k = q.sxz_p;
        syz_k = q.syz_p;
    }
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
__global__ void __launch_bounds__(split_max_threads<T>()) k_velocity(const StepArgs<T> a, const RecFuse rf)
{
    pdl_trigger();
    pdl_wait();
    if (rf.it_wr && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0)
        *rf.it_wr = *rf.it_rd + 1;  // the next step's counter; this launch reads only it_rd
    const int k0 = blockIdx.z * a.kchunk;
    velocity_column<T, MODEL, DAMP, KAHAN, 1, false, 0, true>(a, blockIdx.x * TX + threadIdx.x,
                                                              blockIdx.y * blockDim.y + threadIdx.y, k0,
                                                              min(k0 + a.kchunk, a.nz), 0, rf);
}

// ---------------------------------------------------------------------------------------------
// Receiver gather (OK4:383-386, ANISO:254-268): traces[r*len + it] = field value after the
// velocity update, widened to FP64.  One CTA; thread 0 advances the step counter last (it_wr =
// it_rd + 1: the same location for the one-pass and wavefront forms, the other of the two
// parity locations for the two-kernel step).
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_record(const StepArgs<T> a, const long long *__restrict__ rec_off, const int *__restrict__ rec_comp,
                         int nrec, double *__restrict__ traces, int trace_len, const int *it_rd, int *it_wr)
{
    pdl_trigger();
    pdl_wait();
    const int it = *it_rd;
    if (it >= 0 && it < trace_len)
        for (int r = threadIdx.x; r < nrec; r += blockDim.x)
            traces[(long long)r * trace_len + it] = (double)a.f[rec_comp[r]][rec_off[r]];
    __syncthreads();
    if (threadIdx.x == 0) *it_wr = it + 1;
}

// ---------------------------------------------------------------------------------------------
// Layout conversion between the reference layout (x fastest, the array's own extents) and the
// box layout, with dtype conversion.
// ---------------------------------------------------------------------------------------------
template <typename TD, typename TS>
__global__ void k_pack(TD *__restrict__ box, const TS *__restrict__ src, int ex, int ey, int ez, int sx, long long sy)
{
    const long long n = (long long)ex * ey * ez;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % ex);
        const long long r = e / ex;
        const int j = (int)(r % ey);
        const int k = (int)(r / ey);
        box[(long long)i + (long long)j * sx + (long long)k * sy] = (TD)src[e];
    }
}

template <typename TD, typename TS>
__global__ void k_unpack(TD *__restrict__ dst, const TS *__restrict__ box, int ex, int ey, int ez, int sx, long long sy)
{
    const long long n = (long long)ex * ey * ez;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % ex);
        const long long r = e / ex;
        const int j = (int)(r % ey);
        const int k = (int)(r / ey);
        dst[e] = (TD)box[(long long)i + (long long)j * sx + (long long)k * sy];
    }
}

}  // namespace ewf
