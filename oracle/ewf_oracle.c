/*
 * ewf_oracle.c -- CPU oracle for the staggered-grid elastic FDTD time loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, as plain C loops, the reference solver's
 * time step so that the CUDA product can be checked against it.  It is imported only by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg; the product library
 * never links or calls it.
 *
 * What it restates (file:line within the reference project):
 *   isotropic stress + 1-D PML      src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_OK4_final/FastWaveED_GPU3D_v1.cu:285-331
 *   moment-tensor injection         same file :336-342 (before BC1) and
 *                                   src/FastWaveED_GPU3D_v1_9km_station_ANISO/FastWaveED_GPU3D_v1_9kmst_ANISO.cu:228-252 (after BC1)
 *   free surface BC1                OK4 :271-283, ANISO :270-285 (left out by the two diff_BC schemes)
 *   plane-1 shear modulus           src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_diff_BC2_OK3/FastWaveED_GPU3D_v1.cu:309-323
 *   isotropic velocity update       OK4 :346-378
 *   orthorhombic stress update      ANISO :287-356
 *   orthorhombic velocity update    ANISO :358-389
 *   isotropic stress with edge shear moduli and staggered buoyancy (the 9 km station scheme)
 *                                   src/FastWaveED_GPU3D_v1_9km_station/FastWaveED_GPU3D_v1_9kmst.cu:287-331;
 *                                   its velocity update is ANISO's (9kmst.cu:333-388)
 *   linear velocity damping         src/FastWaveED_GPU3D_v1_16km_station/FastWaveED_GPU3D_v1_16kmst.cu:337-349
 *   per-component 3-D weights       src/FastWaveED_GPU3D_v1_DC_Earthquake/FastWaveED_GPU3D_v1.cu:298-320 (stress),
 *                                   :328-360 (velocity)
 *   receiver sampling               OK4 :383-386, ANISO :254-268
 *   time-loop order                 OK4 :485-505, ANISO :519-555
 *
 * Parity is pinned by tests/golden fixtures that the reference kernels themselves produced
 * (compiled from the reference sources, run on a GPU; see oracle/refkernels.c and
 * tests/golden/make_golden.py).  With -ffp-contract=off the float instantiation matches the
 * reference's FMA-free build bit for bit.
 *
 * Build: see oracle/build.py (gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC).
 */
#include <stddef.h>
#include <stdint.h>

typedef struct orc_grid {
    int32_t nx, ny, nz;
    int32_t model;     /* 0 = isotropic (OK4 scheme), 1 = orthorhombic (ANISO scheme), 2 = 9 km scheme */
    int32_t src_order; /* 0 = injection before BC1 (OK4), 1 = after BC1 (ANISO) */
    int32_t bc1_rows;  /* rows j < bc1_rows get the szz/sxz free-surface rule (OK4:279-281 guard iy<nx) */
    double dx, dy, dz, dt;
    double c66;        /* isotropic shear modulus, scalar pa2[7] (OK4:405) */
    double bx, by, bz; /* isotropic buoyancy 1/rho, scalars pa3[0..2] (OK4:407) */
    double vdamp;      /* linear velocity damping (16 km scheme), 0 = off */
    double c44, c55;   /* per-component-weight scheme: shear moduli of yz and xz (c66: xy) */
    int32_t damping;   /* 3 = per-component weights (w[0..5]: Vx/sxx, Vy/syy, Vz/szz, sxy, sxz, syz) */
    int32_t no_bc1;    /* 1 = no BC1 (the diff_BC schemes: ..._diff_BC_OK2/FastWaveED_GPU3D_v1.cu:453,
                        * ..._diff_BC2_OK3/FastWaveED_GPU3D_v1.cu:476 comment its launch out) */
    double smu;        /* > 0: the isotropic scheme's shear modulus on plane k = 1
                        * (..._diff_BC2_OK3/FastWaveED_GPU3D_v1.cu:309-314, c44u = 1e-5 there) */
} orc_grid;

#define OT float
#define OSUF f32
#include "ewf_oracle_body.h"
#undef OT
#undef OSUF

#define OT double
#define OSUF f64
#include "ewf_oracle_body.h"
#undef OT
#undef OSUF

int orc_abi_version(void) { return 4; }

int orc_num_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
