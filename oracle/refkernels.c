/*
 * refkernels.c -- launcher for the reference's own kernels (TEST INFRASTRUCTURE ONLY).
 *
 * oracle/build.py compiles the reference solvers' device code, unmodified and from where the
 * sources lie in the reference tree, into cubins under oracle/_ref/ (device code only; no host
 * code of the reference is built).  This small library loads such a cubin with the CUDA driver
 * API and launches a kernel by name prefix with an argument vector, so that a Python harness
 * (tests/refrun.py) can replay the reference's time loop (OK4:485-505 / ANISO:519-555) on the
 * same inputs as the product and the CPU oracle.  It is the checker's tool: the product never
 * loads it.
 *
 * libcuda is opened with dlopen so the library builds without the driver stub.
 */
#include <dlfcn.h>
#include <stdio.h>
#include <string.h>

typedef int CUresult;
typedef int CUdevice;
typedef void *CUcontext;
typedef void *CUmodule;
typedef void *CUfunction;
typedef void *CUstream;

static void *g_lib;
static CUresult (*p_cuInit)(unsigned);
static CUresult (*p_cuDeviceGet)(CUdevice *, int);
static CUresult (*p_cuDevicePrimaryCtxRetain)(CUcontext *, CUdevice);
static CUresult (*p_cuCtxSetCurrent)(CUcontext);
static CUresult (*p_cuModuleLoad)(CUmodule *, const char *);
static CUresult (*p_cuModuleUnload)(CUmodule);
static CUresult (*p_cuModuleGetFunctionCount)(unsigned *, CUmodule);
static CUresult (*p_cuModuleEnumerateFunctions)(CUfunction *, unsigned, CUmodule);
static CUresult (*p_cuFuncGetName)(const char **, CUfunction);
static CUresult (*p_cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                                    CUstream, void **, void **);
static CUresult (*p_cuCtxSynchronize)(void);
static CUresult (*p_cuGetErrorString)(CUresult, const char **);

static char g_msg[512];

const char *refk_error(void) { return g_msg; }

static int err(CUresult r, const char *what)
{
    const char *s = "?";
    if (p_cuGetErrorString) p_cuGetErrorString(r, &s);
    snprintf(g_msg, sizeof(g_msg), "%s: CUDA driver error %d (%s)", what, r, s ? s : "?");
    return -(r ? r : 1);
}

int refk_init(int device)
{
    if (!g_lib) {
        g_lib = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!g_lib) g_lib = dlopen("libcuda.so", RTLD_NOW | RTLD_LOCAL);
        if (!g_lib) { snprintf(g_msg, sizeof(g_msg), "dlopen libcuda: %s", dlerror()); return -1; }
#define SYM(name, ver)                                                                        \
        *(void **)&p_##name = dlsym(g_lib, ver);                                              \
        if (!p_##name) { snprintf(g_msg, sizeof(g_msg), "missing driver symbol %s", ver); return -1; }
        SYM(cuInit, "cuInit")
        SYM(cuDeviceGet, "cuDeviceGet")
        SYM(cuDevicePrimaryCtxRetain, "cuDevicePrimaryCtxRetain")
        SYM(cuCtxSetCurrent, "cuCtxSetCurrent")
        SYM(cuModuleLoad, "cuModuleLoad")
        SYM(cuModuleUnload, "cuModuleUnload")
        SYM(cuModuleGetFunctionCount, "cuModuleGetFunctionCount")
        SYM(cuModuleEnumerateFunctions, "cuModuleEnumerateFunctions")
        SYM(cuFuncGetName, "cuFuncGetName")
        SYM(cuLaunchKernel, "cuLaunchKernel")
        SYM(cuCtxSynchronize, "cuCtxSynchronize")
        SYM(cuGetErrorString, "cuGetErrorString")
#undef SYM
    }
    CUresult r = p_cuInit(0);
    if (r) return err(r, "cuInit");
    CUdevice dev;
    if ((r = p_cuDeviceGet(&dev, device))) return err(r, "cuDeviceGet");
    CUcontext ctx;
    if ((r = p_cuDevicePrimaryCtxRetain(&ctx, dev))) return err(r, "cuDevicePrimaryCtxRetain");
    if ((r = p_cuCtxSetCurrent(ctx))) return err(r, "cuCtxSetCurrent");
    return 0;
}

int refk_load(const char *path, void **module)
{
    CUresult r = p_cuModuleLoad((CUmodule *)module, path);
    return r ? err(r, path) : 0;
}

int refk_unload(void *module)
{
    CUresult r = p_cuModuleUnload((CUmodule)module);
    return r ? err(r, "cuModuleUnload") : 0;
}

/* Finds the kernel whose (mangled) name starts with `prefix`, e.g. "_Z17compute_StressPrf". */
int refk_function(void *module, const char *prefix, void **func)
{
    unsigned n = 0;
    CUresult r = p_cuModuleGetFunctionCount(&n, (CUmodule)module);
    if (r) return err(r, "cuModuleGetFunctionCount");
    CUfunction fs[64];
    if (n > 64) n = 64;
    if ((r = p_cuModuleEnumerateFunctions(fs, n, (CUmodule)module))) return err(r, "cuModuleEnumerateFunctions");
    const size_t lp = strlen(prefix);
    for (unsigned i = 0; i < n; ++i) {
        const char *name = NULL;
        if (p_cuFuncGetName(&name, fs[i]) == 0 && name && strncmp(name, prefix, lp) == 0) {
            *func = fs[i];
            return 0;
        }
    }
    snprintf(g_msg, sizeof(g_msg), "no kernel with prefix %s", prefix);
    return -2;
}

int refk_launch(void *func, unsigned gx, unsigned gy, unsigned gz, unsigned bx, unsigned by, unsigned bz, void **args)
{
    CUresult r = p_cuLaunchKernel((CUfunction)func, gx, gy, gz, bx, by, bz, 0, NULL, args, NULL);
    return r ? err(r, "cuLaunchKernel") : 0;
}

int refk_sync(void)
{
    CUresult r = p_cuCtxSynchronize();
    return r ? err(r, "cuCtxSynchronize") : 0;
}
