// ewfd.cu -- host side of libewfd.so: handle, device memory, the time loop under CUDA graphs.
//
// Replaces the reference executable's main() (OK4:390-559, ANISO:391-608): instead of
// compile-time grids, fixed file names and a launch + cudaDeviceSynchronize per kernel
// (OK4:487-498), a handle owns the fields in the padded box layout, a stream, and a CUDA graph
// that replays `graph_steps` time steps per launch; the step index lives on the device so the
// same graph serves every chunk.
#include "ewfd.h"
#include "ewfd_internal.h"
#include "ewfd_kernels.cuh"
#include "ewfd_fused.cuh"
#include "ewfd_band.h"
#include "ewfd_staged.h"
#include "ewfd_wave.cuh"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <type_traits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace ewf;

// ------------------------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------------------------
static thread_local char g_err[512];

int ewf_fail(int status, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return status;
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return ewf_fail(e_ == cudaErrorMemoryAllocation ? EWF_ERR_NOMEM : EWF_ERR_CUDA,          \
                            "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
    } while (0)

extern "C" const char *ewf_last_error(void) { return g_err; }

extern "C" int ewf_abi_version(void) { return EWF_ABI_VERSION; }

extern "C" const char *ewf_strerror(int s)
{
    switch (s) {
    case EWF_OK: return "ok";
    case EWF_ERR_ARG: return "invalid argument";
    case EWF_ERR_CUDA: return "CUDA error";
    case EWF_ERR_NOMEM: return "out of memory";
    case EWF_ERR_IO: return "file I/O error";
    case EWF_ERR_STATE: return "call out of order";
    case EWF_ERR_CFL: return "time step above the CFL limit";
    case EWF_ERR_NONFINITE: return "non-finite values in the receiver traces";
    case EWF_ERR_UNSUPPORTED: return "unsupported configuration";
    case EWF_ERR_NODEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

extern "C" void ewf_params_default(ewf_params *p)
{
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->model = EWF_MODEL_ISO;
    p->precision = EWF_PREC_F32;
    p->damping = EWF_DAMP_PML1D;
    p->src_order = EWF_SRC_BEFORE_BC1;
    p->check_finite = 1;
    p->fused = 0;
    p->free_surface = EWF_FS_BC1;
    p->surface_mu = 0.0;
    p->dx = p->dy = p->dz = 1.0;
    p->dt = 1.0;
}

// ------------------------------------------------------------------------------------------
// geometry helpers
// ------------------------------------------------------------------------------------------
// Extents (reference layout) of a field id; returns false for unknown ids.
bool ewf_field_extent(const ewf_params &p, int id, int *ex, int *ey, int *ez)
{
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    int x = nx, y = ny, z = nz;
    switch (id) {
    case EWF_F_VX: case EWF_M_BX: x = nx + 1; break;
    case EWF_F_VY: case EWF_M_BY: y = ny + 1; break;
    case EWF_F_VZ: case EWF_M_BZ: z = nz + 1; break;
    case EWF_F_SXX: case EWF_F_SYY: case EWF_F_SZZ: break;
    case EWF_F_SXY: case EWF_M_C66XY: x = nx + 1; y = ny + 1; break;
    case EWF_F_SXZ: case EWF_M_C55XZ: x = nx + 1; z = nz + 1; break;
    case EWF_F_SYZ: case EWF_M_C44YZ: y = ny + 1; z = nz + 1; break;
    case EWF_M_C11: case EWF_M_C12: break;
    case EWF_M_C22: case EWF_M_C33: case EWF_M_C13: case EWF_M_C23:
        if (p.model != EWF_MODEL_ORTHO) return false;  // the 9 km scheme has c11/c12 only
        break;
    case EWF_D_WX: x = nx + (p.damping == EWF_DAMP_PML1D ? 1 : 0); y = 1; z = 1; break;
    case EWF_D_WY: x = ny + (p.damping == EWF_DAMP_PML1D ? 1 : 0); y = 1; z = 1; break;
    case EWF_D_WZ: x = nz + (p.damping == EWF_DAMP_PML1D ? 1 : 0); y = 1; z = 1; break;
    case EWF_D_W3D: break;
    case EWF_D_PX: case EWF_D_PXY: case EWF_D_PXZ: case EWF_D_PY: case EWF_D_PYZ: case EWF_D_PZ: {
        if (p.damping != EWF_DAMP_PERCOMP) return false;
        static const int ax[6] = {1, 0, 0, 1, 1, 0}, ay[6] = {0, 1, 0, 1, 0, 1}, az[6] = {0, 0, 1, 0, 1, 1};
        const int q = id - EWF_D_PX;
        x = nx + ax[q]; y = ny + ay[q]; z = nz + az[q];
        break;
    }
    default: return false;
    }
    if ((id == EWF_M_C66XY || id == EWF_M_C55XZ || id == EWF_M_C44YZ || id == EWF_M_BX || id == EWF_M_BY ||
         id == EWF_M_BZ) && p.model == EWF_MODEL_ISO)
        return false;
    if ((id == EWF_D_WX || id == EWF_D_WY || id == EWF_D_WZ) &&
        (p.damping == EWF_DAMP_W3D || p.damping == EWF_DAMP_PERCOMP))
        return false;
    if (id == EWF_D_W3D && p.damping != EWF_DAMP_W3D) return false;
    *ex = x; *ey = y; *ez = z;
    return true;
}

// material slot of a field id (index into m[]), -1 if not a material
static int material_slot(int model, int id)
{
    if (model == EWF_MODEL_ISO) {
        if (id == EWF_M_C11) return 0;
        if (id == EWF_M_C12) return 1;
        return -1;
    }
    if (model == EWF_MODEL_ISO_HET && (id == EWF_M_C22 || id == EWF_M_C33 || id == EWF_M_C13 || id == EWF_M_C23))
        return -1;
    switch (id) {
    case EWF_M_C11: return 0;
    case EWF_M_C22: return 1;
    case EWF_M_C33: return 2;
    case EWF_M_C12: return 3;
    case EWF_M_C13: return 4;
    case EWF_M_C23: return 5;
    case EWF_M_C66XY: return 6;
    case EWF_M_C55XZ: return 7;
    case EWF_M_C44YZ: return 8;
    case EWF_M_BX: return 9;
    case EWF_M_BY: return 10;
    case EWF_M_BZ: return 11;
    default: return -1;
    }
}

static int n_materials(int model) { return model == EWF_MODEL_ISO ? 2 : 12; }
// does this model use material slot q (the 9 km scheme leaves C22, C33, C13, C23 out)
static bool slot_used(int model, int q)
{
    if (q >= n_materials(model)) return false;
    return !(model == EWF_MODEL_ISO_HET && (q == 1 || q == 2 || q == 4 || q == 5));
}

// ------------------------------------------------------------------------------------------
// handle
// ------------------------------------------------------------------------------------------
struct ewf_handle {
    ewf_params p;
    std::string workdir;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t esz = 4;
    int hx = 0, sx = 0;
    long long sy = 0;
    size_t box_elems = 0;
    long long base_off = 0;  // element offset of (0,0,0) inside an allocation
    void *f_alloc[9] = {};
    void *g_alloc[9] = {};  // second state buffer of the fused step
    bool fused = false;
    int onepass = EWF_ONEPASS_TILE;  // one-pass step: its kernel (k_step, k_band with 4 / 8 rows, k_staged)
    StagedPlan *splan = nullptr;     // tensor maps of the staged kernel (encoded on first use)
    bool dbuf = false;      // double-buffered state (one-pass step)
    int flip = 0;           // double-buffered: the current state is in g_alloc when 1
    bool wave = false;      // wavefront step (ewfd_wave.cuh)
    int nsm = 0;            // multiprocessors of the device
    WaveCtl *d_wctl = nullptr;
    int *d_wdone = nullptr;     // done flags, one per stress item
    int wdone_cap = 0;
    int *d_woff = nullptr;      // source entries grouped by owning stress item (n + 1 offsets)
    SrcEntry *d_wsrc = nullptr;
    int woff_cap = 0;
    int wave_key[3] = {-1, -1, -1};  // (kslab, src_version, n) the grouping was built for
    int src_version = 0;
    int wave_lag_pct = 100;     // lag = ntx + 1 + CTAs * pct / 100 (autotuned)
    int wave_hold = -1;         // diagnostic: stress item whose done flag is withheld
    void *comp_alloc[3] = {};
    void *m_alloc[12] = {};
    bool m_set[12] = {};
    void *w1[3] = {};
    bool w_set[10] = {};       // WX WY WZ W3D, then PX PY PZ PXY PXZ PYZ
    void *w3_alloc = nullptr;
    void *w6_alloc[6] = {};    // PERCOMP weight fields
    double *d_stf = nullptr;
    size_t nstf = 0;
    SrcEntry *d_src = nullptr;
    int nsrc = 0;
    std::vector<SrcEntry> h_src;
    StressSrc src_fuse{};   // two-kernel step: the sources the stress kernel applies (nsrc 0: k_inject does)
    long long *d_rec_off = nullptr;
    int *d_rec_comp = nullptr;
    int nrec = 0;
    std::vector<int32_t> h_rec;  // n*4 (i,j,k,comp)
    double *d_traces = nullptr;
    int *d_it = nullptr;     // step counter: [0] (one-pass, wavefront forms); [it & 1] (two-kernel step)
    int *d_rcol = nullptr;   // two-kernel step: first receiver entry per column (nx*ny, -1 none)
    int4 *d_rent = nullptr;  // its entries: (k, component, trace row, next entry)
    bool rec_fuse = true;    // the velocity kernel samples every receiver (else k_record does)
    int it = 0;
    void *d_stage = nullptr;
    size_t stage_bytes = 0;
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 0;
    bool graph_dirty = true;
    float last_ms = 0.f;
    int kchunk = 32;
    int ty = TY;        // two-kernel step: CTA tile height in rows (autotuned)
    bool pdl = true;    // two-kernel step: kernels launched as programmatic dependents (off if capture refuses)
    int l2pf = 0;       // two-kernel step: L2 prefetch distance of the velocity kernel in planes (autotuned)
    bool fdiv = false;  // div_spacing verified for (float) dx, dy, dz
    struct Snapshots *snap = nullptr;  // queued snapshot writer (created on first use)
};

// ------------------------------------------------------------------------------------------
// queued snapshots: device copy in stream order, D2H on a second stream, files by a thread
// ------------------------------------------------------------------------------------------
struct Snapshots {
    struct Slot {
        void *dev = nullptr;          // Vx | Vy | Vz in the reference layout
        void *host = nullptr;         // pinned
        cudaEvent_t ready = nullptr;  // device copy done (solver stream)
        cudaEvent_t done = nullptr;   // D2H done (copy stream)
        bool busy = false;
        int isave = 0;
    };
    int device = 0;
    size_t n[3] = {0, 0, 0};
    size_t esz = 4;
    std::string dir;
    cudaStream_t copy = nullptr;
    Slot slot[2];
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> queue;  // slots whose files are still to be written, oldest first
    bool stop = false;
    int error = EWF_OK;
    std::string error_msg;
    std::thread worker;

    void run()
    {
        cudaSetDevice(device);
        for (;;) {
            int q;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                q = queue.front();
            }
            Slot &sl = slot[q];
            int st = EWF_OK;
            std::string msg;
            if (cudaEventSynchronize(sl.done) != cudaSuccess) {
                st = EWF_ERR_CUDA;
                msg = "snapshot copy failed";
                cudaGetLastError();
            } else {
                static const char *names[3] = {"Vx", "Vy", "Vz"};
                const char *base = (const char *)sl.host;
                for (int f = 0; f < 3 && st == EWF_OK; ++f) {
                    char fn[64];
                    snprintf(fn, sizeof(fn), "/%d_0_%s.res", sl.isave, names[f]);
                    st = ewf_write_raw_file((dir + fn).c_str(), base, n[f] * esz);
                    if (st) msg = ewf_last_error();
                    base += n[f] * esz;
                }
            }
            std::lock_guard<std::mutex> lk(mu);
            if (st && error == EWF_OK) {
                error = st;
                error_msg = msg;
            }
            sl.busy = false;
            queue.pop_front();
            cv.notify_all();
        }
    }
};

static void snapshots_close(ewf_handle *h)
{
    Snapshots *S = h->snap;
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto &sl : S->slot) {
        if (sl.dev) cudaFree(sl.dev);
        if (sl.host) cudaFreeHost(sl.host);
        if (sl.ready) cudaEventDestroy(sl.ready);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    if (S->copy) cudaStreamDestroy(S->copy);
    delete S;
    h->snap = nullptr;
}

static void *boxptr(const ewf_handle *h, void *alloc)
{
    return alloc ? (void *)((char *)alloc + h->base_off * (long long)h->esz) : nullptr;
}

// state buffer `which` (0: f_alloc, 1: g_alloc)
static void *state_alloc(const ewf_handle *h, int which, int q) { return which ? h->g_alloc[q] : h->f_alloc[q]; }

template <typename T>
static StepArgs<T> make_args(const ewf_handle *h, int which = -1)
{
    if (which < 0) which = h->flip;
    StepArgs<T> a;
    memset(&a, 0, sizeof(a));
    for (int q = 0; q < 9; ++q) a.f[q] = (T *)boxptr(h, state_alloc(h, which, q));
    for (int q = 0; q < 3; ++q) a.comp[q] = (T *)boxptr(h, h->comp_alloc[q]);
    for (int q = 0; q < 12; ++q) a.m[q] = (const T *)boxptr(h, h->m_alloc[q]);
    for (int q = 0; q < 3; ++q) a.w1[q] = (const T *)h->w1[q];
    a.w3 = (const T *)boxptr(h, h->w3_alloc);
    for (int q = 0; q < 6; ++q) a.w6[q] = (const T *)boxptr(h, h->w6_alloc[q]);
    a.sy = h->sy;
    a.sx = h->sx;
    a.R = 1;
    a.sxs = h->sx;
    a.sys = h->sy;
    a.nx = h->p.nx;
    a.ny = h->p.ny;
    a.nz = h->p.nz;
    a.bc1_rows = std::min(h->p.nx, h->p.ny + std::max(0, h->p.over_y));
    if (a.bc1_rows > h->p.ny) a.bc1_rows = h->p.ny;
    a.kchunk = h->kchunk;
    // scalar parameters are rounded to T exactly as the reference passes them (const DAT args)
    a.dt = (T)h->p.dt;
    a.dx = (T)h->p.dx;
    a.dy = (T)h->p.dy;
    a.dz = (T)h->p.dz;
    a.rdt = (T)1.0 / a.dt;
    a.rdx = (T)1.0 / a.dx;
    a.rdy = (T)1.0 / a.dy;
    a.rdz = (T)1.0 / a.dz;
    a.c66 = (T)h->p.c66;
    a.c44 = (T)h->p.c44;
    a.c55 = (T)h->p.c55;
    a.bx = (T)h->p.bx;
    a.by = (T)h->p.by;
    a.bz = (T)h->p.bz;
    a.third = (T)1.0 / (T)3.0;
    a.fdiv = h->fdiv ? 1 : 0;
    a.l2pf = h->l2pf;
    a.vdamp = (T)h->p.vdamp;
    a.bc1 = h->p.free_surface == EWF_FS_BC1 ? 1 : 0;
    a.smu_on = h->p.surface_mu > 0.0 ? 1 : 0;
    a.smu = (T)h->p.surface_mu;
    return a;
}

// ------------------------------------------------------------------------------------------
// device check of div_spacing: every significand of three binades of x (2^-90, 2^0, 2^99, both
// signs) against IEEE division; the range argument in ewfd_kernels.cuh carries the result to
// the whole range
// ------------------------------------------------------------------------------------------
namespace ewf {
__global__ void k_fdiv_check(float d, float r, unsigned *bad)
{
    const unsigned m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= (1u << 23)) return;
    const unsigned expo[3] = {37u, 127u, 226u};
    unsigned nbad = 0;
    for (int b = 0; b < 3; ++b)
        for (unsigned sgn = 0; sgn < 2; ++sgn) {
            const float x = __uint_as_float((sgn << 31) | (expo[b] << 23) | m);
            if (__float_as_uint(div_spacing(x, d, r, true)) != __float_as_uint(__fdiv_rn(x, d))) ++nbad;
        }
    if (nbad) atomicAdd(bad, nbad);
}
}  // namespace ewf

bool ewf_fdiv_verified(float d)
{
    if (!(d >= 0x1p-10f && d <= 0x1p30f)) return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    uint32_t bits;
    memcpy(&bits, &d, sizeof(bits));
    static std::mutex mu;
    static std::map<std::pair<int, uint32_t>, bool> cache;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(dev, bits);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    unsigned *dbad = nullptr, hbad = 1;
    cudaStream_t st = nullptr;
    bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&dbad, sizeof(unsigned)) == cudaSuccess &&
              cudaMemsetAsync(dbad, 0, sizeof(unsigned), st) == cudaSuccess;
    if (ok) {
        k_fdiv_check<<<(1u << 23) / 256, 256, 0, st>>>(d, 1.0f / d, dbad);
        ok = cudaGetLastError() == cudaSuccess &&
             cudaMemcpyAsync(&hbad, dbad, sizeof(unsigned), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (dbad) cudaFree(dbad);
    if (st) cudaStreamDestroy(st);
    cudaGetLastError();
    ok = ok && hbad == 0;
    cache[key] = ok;
    return ok;
}

static int dev_zero(ewf_handle *h, void *alloc)
{
    if (alloc) CK(cudaMemsetAsync(alloc, 0, h->box_elems * h->esz, h->stream));
    return EWF_OK;
}

static int alloc_box(ewf_handle *h, void **out)
{
    CK(cudaMalloc(out, h->box_elems * h->esz));
    CK(cudaMemsetAsync(*out, 0, h->box_elems * h->esz, h->stream));
    return EWF_OK;
}

extern "C" void ewf_destroy(ewf_handle *h)
{
    if (!h) return;
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    snapshots_close(h);  // finishes the queued snapshot files first
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    for (auto &x : h->f_alloc) cudaFree(x);
    for (auto &x : h->g_alloc) cudaFree(x);
    for (auto &x : h->comp_alloc) cudaFree(x);
    for (auto &x : h->m_alloc) cudaFree(x);
    for (auto &x : h->w1) cudaFree(x);
    cudaFree(h->w3_alloc);
    for (auto &x : h->w6_alloc) cudaFree(x);
    cudaFree(h->d_stf);
    cudaFree(h->d_src);
    cudaFree(h->d_wctl);
    cudaFree(h->d_wdone);
    cudaFree(h->d_woff);
    cudaFree(h->d_wsrc);
    cudaFree(h->d_rec_off);
    cudaFree(h->d_rec_comp);
    cudaFree(h->d_traces);
    cudaFree(h->d_it);
    cudaFree(h->d_rcol);
    cudaFree(h->d_rent);
    cudaFree(h->d_stage);
    delete h->splan;
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (cur >= 0) cudaSetDevice(cur);
    delete h;
}

static int validate_params(const ewf_params *p)
{
    if (!p) return ewf_fail(EWF_ERR_ARG, "params is NULL");
    if (p->nx < 4 || p->ny < 4 || p->nz < 4)
        return ewf_fail(EWF_ERR_ARG, "grid %dx%dx%d: every extent must be >= 4", p->nx, p->ny, p->nz);
    if ((long long)p->nx * p->ny * p->nz > (1LL << 36)) return ewf_fail(EWF_ERR_ARG, "grid too large");
    if (p->nt < 1) return ewf_fail(EWF_ERR_ARG, "nt must be >= 1 (got %d)", p->nt);
    if (p->model < EWF_MODEL_ISO || p->model > EWF_MODEL_ISO_HET) return ewf_fail(EWF_ERR_ARG, "unknown model %d", p->model);
    if (p->precision < EWF_PREC_F32 || p->precision > EWF_PREC_F64) return ewf_fail(EWF_ERR_ARG, "unknown precision %d", p->precision);
    if (p->model == EWF_MODEL_ISO && p->damping != EWF_DAMP_PML1D && p->damping != EWF_DAMP_PERCOMP)
        return ewf_fail(EWF_ERR_UNSUPPORTED, "the isotropic scheme uses 1-D PML profiles or per-component weights (damping 0 or 3)");
    if (p->fused < EWF_STEP_SPLIT || p->fused > EWF_STEP_WAVE) return ewf_fail(EWF_ERR_ARG, "unknown step form %d", p->fused);
    if (p->damping == EWF_DAMP_PERCOMP && (p->model != EWF_MODEL_ISO || p->fused == EWF_STEP_FUSED))
        return ewf_fail(EWF_ERR_UNSUPPORTED, "per-component weights: isotropic model, two-kernel or wavefront step");
    if (p->model != EWF_MODEL_ISO && p->damping != EWF_DAMP_W3D && p->damping != EWF_DAMP_SEPARABLE)
        return ewf_fail(EWF_ERR_UNSUPPORTED, "the orthorhombic and 9 km schemes use a 3-D or separable weight field (damping 1 or 2)");
    if (p->model == EWF_MODEL_ISO_HET && p->fused == EWF_STEP_FUSED)
        return ewf_fail(EWF_ERR_UNSUPPORTED, "the one-pass step is built for models 0 and 1");
    if (!(p->vdamp >= 0.0) || p->vdamp >= 1.0) return ewf_fail(EWF_ERR_ARG, "vdamp must be in [0, 1)");
    if (p->vdamp != 0.0 && (p->model == EWF_MODEL_ISO || p->precision == EWF_PREC_F32_KAHAN || p->fused == EWF_STEP_FUSED))
        return ewf_fail(EWF_ERR_UNSUPPORTED, "vdamp applies to models 1 and 2 in FP32/FP64 with the two-kernel or wavefront step");
    if (p->src_order != EWF_SRC_BEFORE_BC1 && p->src_order != EWF_SRC_AFTER_BC1)
        return ewf_fail(EWF_ERR_ARG, "unknown src_order %d", p->src_order);
    if (p->over_y < 0) return ewf_fail(EWF_ERR_ARG, "over_y must be >= 0");
    if (p->nx > p->ny && p->over_y > 0)
        return ewf_fail(EWF_ERR_UNSUPPORTED,
                        "nx > ny with over_y > 0: the reference free-surface kernel writes rows past ny into the next "
                        "plane while other threads read it (a race); no defined result to reproduce");
    if (!(p->dx > 0 && p->dy > 0 && p->dz > 0 && p->dt > 0)) return ewf_fail(EWF_ERR_ARG, "dx, dy, dz, dt must be > 0");
    if (p->kchunk != 0 && p->kchunk < 4) return ewf_fail(EWF_ERR_ARG, "kchunk must be 0 or >= 4");
    if (p->free_surface != EWF_FS_BC1 && p->free_surface != EWF_FS_NONE)
        return ewf_fail(EWF_ERR_ARG, "unknown free_surface %d", p->free_surface);
    if (!(p->surface_mu >= 0.0)) return ewf_fail(EWF_ERR_ARG, "surface_mu must be >= 0");
    if (p->surface_mu > 0.0 && (p->model != EWF_MODEL_ISO || p->damping != EWF_DAMP_PML1D))
        return ewf_fail(EWF_ERR_UNSUPPORTED, "surface_mu applies to the isotropic scheme with 1-D PML profiles "
                                             "(the other schemes take the layer in their edge shear-modulus fields)");
    if ((p->free_surface != EWF_FS_BC1 || p->surface_mu > 0.0) && p->fused == EWF_STEP_FUSED)
        return ewf_fail(EWF_ERR_UNSUPPORTED, "the one-pass step applies BC1 and the plain shear modulus only");
    return EWF_OK;
}

static bool band_fits(const ewf_handle *h, int rows);
// rows per CTA of the band kernel for a one-pass kernel choice (0: not the band kernel)
static int band_rows(int onepass) { return onepass == EWF_ONEPASS_BAND4 ? 4 : (onepass == EWF_ONEPASS_BAND8 ? 8 : 0); }

extern "C" int ewf_create(const ewf_params *p, ewf_handle **out)
{
    if (!out) return ewf_fail(EWF_ERR_ARG, "out is NULL");
    *out = nullptr;
    int st = validate_params(p);
    if (st) return st;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return ewf_fail(EWF_ERR_NODEVICE, "no CUDA device visible");
    }
    ewf_handle *h = new (std::nothrow) ewf_handle();
    if (!h) return ewf_fail(EWF_ERR_NOMEM, "host allocation");
    h->p = *p;
    h->workdir = p->workdir ? p->workdir : ".";
    h->p.workdir = nullptr;
    cudaGetDevice(&h->device);
    h->esz = (p->precision == EWF_PREC_F64) ? 8 : 4;
    h->hx = (int)(128 / h->esz);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    h->sx = h->hx + ((nx + 2 + 31) / 32) * 32;
    const long long py = ny + 3, pz = nz + 3;
    h->sy = (long long)h->sx * py;
    h->box_elems = (size_t)h->sy * pz;
    h->base_off = h->hx + (long long)h->sx * 1 + h->sy * 1;
    h->kchunk = p->kchunk > 0 ? p->kchunk : 16;
    h->gsteps = p->graph_steps == 0 ? 64 : (p->graph_steps < 0 ? 0 : p->graph_steps);
    if ((p->fused == EWF_STEP_FUSED || p->fused == EWF_STEP_SPLIT) && (h->gsteps & 1))
        h->gsteps += 1;  // graphs replay buffer pairs (one-pass) / step-counter pairs (two-kernel step)

#define CKH(call)                                                                                    \
    do {                                                                                             \
        int s_ = (call);                                                                             \
        if (s_) { ewf_destroy(h); return s_; }                                                       \
    } while (0)
#define CKC(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            int s_ = ewf_fail(e_ == cudaErrorMemoryAllocation ? EWF_ERR_NOMEM : EWF_ERR_CUDA,         \
                              "%s: %s", #call, cudaGetErrorString(e_));                              \
            ewf_destroy(h);                                                                          \
            return s_;                                                                               \
        }                                                                                            \
    } while (0)

    CKC(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&h->ev0));
    CKC(cudaEventCreate(&h->ev1));
    h->fused = p->fused == EWF_STEP_FUSED;
    h->wave = p->fused == EWF_STEP_WAVE;
    h->dbuf = h->fused;
    CKC(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
    if (h->wave) {
        CKC(cudaMalloc(&h->d_wctl, sizeof(WaveCtl)));
        CKC(cudaMemsetAsync(h->d_wctl, 0, sizeof(WaveCtl), h->stream));
    }
    if (p->model == EWF_MODEL_ORTHO && h->esz == 4)
        h->fdiv = ewf_fdiv_verified((float)p->dx) && ewf_fdiv_verified((float)p->dy) && ewf_fdiv_verified((float)p->dz);
    for (int q = 0; q < 9; ++q) CKH(alloc_box(h, &h->f_alloc[q]));
    if (h->dbuf)
        for (int q = 0; q < 9; ++q) CKH(alloc_box(h, &h->g_alloc[q]));
    if (p->precision == EWF_PREC_F32_KAHAN)
        for (int q = 0; q < 3; ++q) CKH(alloc_box(h, &h->comp_alloc[q]));
    for (int q = 0; q < n_materials(p->model); ++q)
        if (slot_used(p->model, q)) CKH(alloc_box(h, &h->m_alloc[q]));
    if (p->damping == EWF_DAMP_W3D) {
        CKH(alloc_box(h, &h->w3_alloc));
    } else if (p->damping == EWF_DAMP_PERCOMP) {
        for (int q = 0; q < 6; ++q) CKH(alloc_box(h, &h->w6_alloc[q]));
    } else {
        const int n1[3] = {nx + 1, ny + 1, nz + 1};
        for (int q = 0; q < 3; ++q) {
            CKC(cudaMalloc(&h->w1[q], (size_t)(n1[q] + 1) * h->esz));
            CKC(cudaMemsetAsync(h->w1[q], 0, (size_t)(n1[q] + 1) * h->esz, h->stream));
        }
    }
    CKC(cudaMalloc(&h->d_it, 2 * sizeof(int)));
    CKC(cudaMemsetAsync(h->d_it, 0, 2 * sizeof(int), h->stream));
    // staging buffer for host transfers in the reference layout (largest field, FP64)
    h->stage_bytes = (size_t)(nx + 1) * (ny + 1) * (nz + 1) * 8;
    CKC(cudaMalloc(&h->d_stage, h->stage_bytes));
    CKC(cudaStreamSynchronize(h->stream));
#undef CKH
#undef CKC
    *out = h;
    return EWF_OK;
}

extern "C" int ewf_get_params(const ewf_handle *h, ewf_params *out)
{
    if (!h || !out) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *out = h->p;
    out->workdir = h->workdir.c_str();
    return EWF_OK;
}

const char *ewf_workdir(const ewf_handle *h) { return h->workdir.c_str(); }
int ewf_nrec(const ewf_handle *h) { return h->nrec; }
int ewf_esz(const ewf_handle *h) { return (int)h->esz; }
const double *ewf_stf_host_copy(const ewf_handle *h, std::vector<double> &out)
{
    out.resize(h->nstf);
    if (h->nstf) cudaMemcpy(out.data(), h->d_stf, h->nstf * sizeof(double), cudaMemcpyDeviceToHost);
    return out.data();
}

extern "C" size_t ewf_field_size(const ewf_handle *h, int32_t field)
{
    if (!h) return 0;
    int ex, ey, ez;
    if (!ewf_field_extent(h->p, field, &ex, &ey, &ez)) return 0;
    return (size_t)ex * ey * ez;
}

// device pointer (box base or 1-D array) of a field id
static void *field_dev(ewf_handle *h, int id, bool *is_box)
{
    *is_box = true;
    if (id >= EWF_F_VX && id <= EWF_F_SYZ) return boxptr(h, state_alloc(h, h->flip, id));
    const int ms = material_slot(h->p.model, id);
    if (ms >= 0) return boxptr(h, h->m_alloc[ms]);
    if (id == EWF_D_W3D) return boxptr(h, h->w3_alloc);
    if (id >= EWF_D_PX && id <= EWF_D_PYZ) return boxptr(h, h->w6_alloc[id - EWF_D_PX]);
    if (id >= EWF_D_WX && id <= EWF_D_WZ) {
        *is_box = false;
        return h->w1[id - EWF_D_WX];
    }
    return nullptr;
}

static unsigned pack_blocks(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16); }

extern "C" int ewf_set_field(ewf_handle *h, int32_t field, const void *host, size_t n, int32_t dtype_bytes)
{
    if (!h || !host) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    if (dtype_bytes != 4 && dtype_bytes != 8) return ewf_fail(EWF_ERR_ARG, "dtype_bytes must be 4 or 8");
    int ex, ey, ez;
    if (!ewf_field_extent(h->p, field, &ex, &ey, &ez))
        return ewf_fail(EWF_ERR_ARG, "field %d does not exist for this model/damping", field);
    const size_t need = (size_t)ex * ey * ez;
    if (n != need) return ewf_fail(EWF_ERR_ARG, "field %d: %zu elements given, %zu expected", field, n, need);
    bool is_box;
    void *dst = field_dev(h, field, &is_box);
    if (!dst) return ewf_fail(EWF_ERR_STATE, "field %d has no storage", field);
    CK(cudaMemcpyAsync(h->d_stage, host, n * dtype_bytes, cudaMemcpyHostToDevice, h->stream));
    const int sx = is_box ? h->sx : 0;
    const long long sy = is_box ? h->sy : 0;
    const unsigned nb = pack_blocks(n);
    if (h->esz == 4) {
        if (dtype_bytes == 4) k_pack<float, float><<<nb, 256, 0, h->stream>>>((float *)dst, (const float *)h->d_stage, ex, ey, ez, sx, sy);
        else k_pack<float, double><<<nb, 256, 0, h->stream>>>((float *)dst, (const double *)h->d_stage, ex, ey, ez, sx, sy);
    } else {
        if (dtype_bytes == 4) k_pack<double, float><<<nb, 256, 0, h->stream>>>((double *)dst, (const float *)h->d_stage, ex, ey, ez, sx, sy);
        else k_pack<double, double><<<nb, 256, 0, h->stream>>>((double *)dst, (const double *)h->d_stage, ex, ey, ez, sx, sy);
    }
    CK(cudaGetLastError());
    if (h->dbuf && field >= EWF_F_VX && field <= EWF_F_SYZ) {
        // both state buffers hold the cells the step never updates
        void *dst2 = boxptr(h, state_alloc(h, 1 - h->flip, field));
        if (h->esz == 4) {
            if (dtype_bytes == 4) k_pack<float, float><<<nb, 256, 0, h->stream>>>((float *)dst2, (const float *)h->d_stage, ex, ey, ez, sx, sy);
            else k_pack<float, double><<<nb, 256, 0, h->stream>>>((float *)dst2, (const double *)h->d_stage, ex, ey, ez, sx, sy);
        } else {
            if (dtype_bytes == 4) k_pack<double, float><<<nb, 256, 0, h->stream>>>((double *)dst2, (const float *)h->d_stage, ex, ey, ez, sx, sy);
            else k_pack<double, double><<<nb, 256, 0, h->stream>>>((double *)dst2, (const double *)h->d_stage, ex, ey, ez, sx, sy);
        }
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(h->stream));
    const int ms = material_slot(h->p.model, field);
    if (ms >= 0) h->m_set[ms] = true;
    if (field >= EWF_D_WX && field <= EWF_D_PYZ) h->w_set[field - EWF_D_WX] = true;
    return EWF_OK;
}

extern "C" int ewf_get_field(ewf_handle *h, int32_t field, void *host, size_t n, int32_t dtype_bytes)
{
    if (!h || !host) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    if (dtype_bytes != 4 && dtype_bytes != 8) return ewf_fail(EWF_ERR_ARG, "dtype_bytes must be 4 or 8");
    int ex, ey, ez;
    if (!ewf_field_extent(h->p, field, &ex, &ey, &ez))
        return ewf_fail(EWF_ERR_ARG, "field %d does not exist for this model/damping", field);
    const size_t need = (size_t)ex * ey * ez;
    if (n != need) return ewf_fail(EWF_ERR_ARG, "field %d: %zu elements given, %zu expected", field, n, need);
    bool is_box;
    void *src = field_dev(h, field, &is_box);
    if (!src) return ewf_fail(EWF_ERR_STATE, "field %d has no storage", field);
    const int sx = is_box ? h->sx : 0;
    const long long sy = is_box ? h->sy : 0;
    const unsigned nb = pack_blocks(n);
    if (h->esz == 4) {
        if (dtype_bytes == 4) k_unpack<float, float><<<nb, 256, 0, h->stream>>>((float *)h->d_stage, (const float *)src, ex, ey, ez, sx, sy);
        else k_unpack<double, float><<<nb, 256, 0, h->stream>>>((double *)h->d_stage, (const float *)src, ex, ey, ez, sx, sy);
    } else {
        if (dtype_bytes == 4) k_unpack<float, double><<<nb, 256, 0, h->stream>>>((float *)h->d_stage, (const double *)src, ex, ey, ez, sx, sy);
        else k_unpack<double, double><<<nb, 256, 0, h->stream>>>((double *)h->d_stage, (const double *)src, ex, ey, ez, sx, sy);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, h->d_stage, n * dtype_bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return EWF_OK;
}

extern "C" int ewf_write_snapshot_async(ewf_handle *h, int32_t isave)
{
    if (!h || isave < 0) return ewf_fail(EWF_ERR_ARG, "bad argument");
    static const int ids[3] = {EWF_F_VX, EWF_F_VY, EWF_F_VZ};
    if (!h->snap) {
        Snapshots *S = new (std::nothrow) Snapshots();
        if (!S) return ewf_fail(EWF_ERR_NOMEM, "host allocation");
        h->snap = S;
        S->device = h->device;
        S->esz = h->esz;
        S->dir = h->workdir;
        size_t total = 0;
        for (int f = 0; f < 3; ++f) total += (S->n[f] = ewf_field_size(h, ids[f]));
        CK(cudaStreamCreateWithFlags(&S->copy, cudaStreamNonBlocking));
        for (auto &sl : S->slot) {
            CK(cudaMalloc(&sl.dev, total * S->esz));
            CK(cudaMallocHost(&sl.host, total * S->esz));
            CK(cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
        }
        S->worker = std::thread([S] { S->run(); });
    }
    Snapshots *S = h->snap;
    int q;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        S->cv.wait(lk, [&] { return !S->slot[0].busy || !S->slot[1].busy; });
        q = S->slot[0].busy ? 1 : 0;
        S->slot[q].busy = true;
        S->slot[q].isave = isave;
    }
    Snapshots::Slot &sl = S->slot[q];
    char *dst = (char *)sl.dev;
    for (int f = 0; f < 3; ++f) {
        int ex, ey, ez;
        ewf_field_extent(h->p, ids[f], &ex, &ey, &ez);
        bool is_box;
        const void *src = field_dev(h, ids[f], &is_box);
        const unsigned nb = pack_blocks(S->n[f]);
        if (h->esz == 4)
            k_unpack<float, float><<<nb, 256, 0, h->stream>>>((float *)dst, (const float *)src, ex, ey, ez, h->sx, h->sy);
        else
            k_unpack<double, double><<<nb, 256, 0, h->stream>>>((double *)dst, (const double *)src, ex, ey, ez, h->sx, h->sy);
        dst += S->n[f] * S->esz;
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(sl.ready, h->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S->copy, sl.ready, 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sl.host, sl.dev, (S->n[0] + S->n[1] + S->n[2]) * S->esz, cudaMemcpyDeviceToHost, S->copy);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, S->copy);
    std::lock_guard<std::mutex> lk(S->mu);
    if (e != cudaSuccess) {
        sl.busy = false;
        S->cv.notify_all();
        return ewf_fail(EWF_ERR_CUDA, "snapshot: %s", cudaGetErrorString(e));
    }
    S->queue.push_back(q);
    S->cv.notify_all();
    return EWF_OK;
}

extern "C" int ewf_snapshot_wait(ewf_handle *h)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    Snapshots *S = h->snap;
    if (!S) return EWF_OK;
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv.wait(lk, [&] { return S->queue.empty(); });
    const int st = S->error;
    if (st) {
        ewf_fail(st, "%s", S->error_msg.c_str());
        S->error = EWF_OK;
    }
    return st;
}

extern "C" int ewf_set_stf(ewf_handle *h, const double *stf, size_t n)
{
    if (!h || (!stf && n)) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    if (n < (size_t)h->p.nt) return ewf_fail(EWF_ERR_ARG, "Src has %zu samples, nt = %d", n, h->p.nt);
    if (n != h->nstf) {
        CK(cudaStreamSynchronize(h->stream));
        cudaFree(h->d_stf);
        h->d_stf = nullptr;
        h->nstf = 0;
        CK(cudaMalloc(&h->d_stf, n * sizeof(double)));
        h->nstf = n;
        h->graph_dirty = true;
    }
    CK(cudaMemcpyAsync(h->d_stf, stf, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return EWF_OK;
}

extern "C" int ewf_set_sources(ewf_handle *h, int32_t n, const int32_t *cijk, const double *coef)
{
    if (!h || n < 0 || (n > 0 && (!cijk || !coef))) return ewf_fail(EWF_ERR_ARG, "bad source list");
    if (n > MAXSRC) return ewf_fail(EWF_ERR_ARG, "%d point sources, at most %d", n, MAXSRC);
    std::vector<SrcEntry> v((size_t)n);
    for (int e = 0; e < n; ++e) {
        const int c = cijk[4 * e], i = cijk[4 * e + 1], j = cijk[4 * e + 2], k = cijk[4 * e + 3];
        if (c < EWF_F_SXX || c > EWF_F_SYZ) return ewf_fail(EWF_ERR_ARG, "source %d: component %d is not a stress field", e, c);
        int ex, ey, ez;
        ewf_field_extent(h->p, c, &ex, &ey, &ez);
        if (i < 0 || j < 0 || k < 0 || i >= ex || j >= ey || k >= ez)
            return ewf_fail(EWF_ERR_ARG, "source %d: cell (%d,%d,%d) outside field %d (%dx%dx%d)", e, i, j, k, c, ex, ey, ez);
        v[e] = SrcEntry{c, i, j, k, coef[e]};
    }
    CK(cudaStreamSynchronize(h->stream));
    if (n > h->nsrc || !h->d_src) {
        cudaFree(h->d_src);
        h->d_src = nullptr;
        if (n > 0) CK(cudaMalloc(&h->d_src, (size_t)n * sizeof(SrcEntry)));
    }
    if (n > 0) CK(cudaMemcpy(h->d_src, v.data(), (size_t)n * sizeof(SrcEntry), cudaMemcpyHostToDevice));
    h->h_src = v;
    h->nsrc = n;
    h->src_version++;
    h->graph_dirty = true;
    // the stress kernel's threads apply the entries when all of them lie in its cells (k_inject
    // covers the rest: cells on the staggered arrays' last planes, and grids too thin for BC1's
    // plane-2 copy)
    StressSrc f{};
    bool fuse = n > 0 && h->p.nz >= 3;
    f.i0 = f.j0 = INT32_MAX;
    f.i1 = f.j1 = f.k1 = -1;
    for (const SrcEntry &q : v) {
        if (q.i >= h->p.nx || q.j >= h->p.ny || q.k >= h->p.nz) fuse = false;
        f.i0 = std::min(f.i0, q.i);
        f.i1 = std::max(f.i1, q.i);
        f.j0 = std::min(f.j0, q.j);
        f.j1 = std::max(f.j1, q.j);
        f.k1 = std::max(f.k1, fused_src_plane(q.comp, q.k));
    }
    if (fuse) {
        f.src = h->d_src;
        f.nsrc = n;
    } else {
        f = StressSrc{};
    }
    h->src_fuse = f;
    return EWF_OK;
}

extern "C" int ewf_set_moment_tensor(ewf_handle *h, const double mt[6], int32_t xs, int32_t ys, int32_t zs, int32_t stencil)
{
    if (!h || !mt) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    // component order of mt: xx yy zz xy xz yz
    int32_t cijk[24];
    double coef[6];
    int n = 0;
    auto add = [&](int comp, int di, int dj, int dk, double c) {
        cijk[4 * n] = comp; cijk[4 * n + 1] = xs + di; cijk[4 * n + 2] = ys + dj; cijk[4 * n + 3] = zs + dk;
        coef[n++] = c;
    };
    if (stencil == 0) {
        // OK4:336-342: normals at (xs+1,ys+1,zs+1), yz at (xs+2,ys+2), xz and xy at (xs+3,ys+3)
        add(EWF_F_SXX, 1, 1, 1, mt[0]);
        add(EWF_F_SYY, 1, 1, 1, mt[1]);
        add(EWF_F_SZZ, 1, 1, 1, mt[2]);
        add(EWF_F_SYZ, 2, 2, 1, mt[5]);
        add(EWF_F_SXZ, 3, 3, 1, mt[4]);
        add(EWF_F_SXY, 3, 3, 1, mt[3]);
    } else if (stencil == 1) {
        // ANISO:233-247: normals at (xs+1,ys+1), xy at (xs+2,ys+2), yz at (xs+3,ys+2), xz at (xs-1,ys+1)
        add(EWF_F_SXX, 1, 1, 1, mt[0]);
        add(EWF_F_SYY, 1, 1, 1, mt[1]);
        add(EWF_F_SZZ, 1, 1, 1, mt[2]);
        add(EWF_F_SXY, 2, 2, 1, mt[3]);
        add(EWF_F_SYZ, 3, 2, 1, mt[5]);
        add(EWF_F_SXZ, -1, 1, 1, mt[4]);
    } else {
        return ewf_fail(EWF_ERR_ARG, "stencil must be 0 (OK4) or 1 (ANISO)");
    }
    return ewf_set_sources(h, n, cijk, coef);
}

extern "C" int ewf_set_receivers(ewf_handle *h, int32_t n, const int32_t *ijkc)
{
    if (!h || n < 0 || (n > 0 && !ijkc)) return ewf_fail(EWF_ERR_ARG, "bad receiver list");
    std::vector<long long> off((size_t)n);
    std::vector<int> comp((size_t)n);
    for (int r = 0; r < n; ++r) {
        const int i = ijkc[4 * r], j = ijkc[4 * r + 1], k = ijkc[4 * r + 2], c = ijkc[4 * r + 3];
        if (c < EWF_F_VX || c > EWF_F_SYZ) return ewf_fail(EWF_ERR_ARG, "receiver %d: field %d is not a state field", r, c);
        int ex, ey, ez;
        ewf_field_extent(h->p, c, &ex, &ey, &ez);
        if (i < 0 || j < 0 || k < 0 || i >= ex || j >= ey || k >= ez)
            return ewf_fail(EWF_ERR_ARG, "receiver %d: cell (%d,%d,%d) outside field %d", r, i, j, k, c);
        off[r] = (long long)i + (long long)j * h->sx + (long long)k * h->sy;
        comp[r] = c;
    }
    CK(cudaStreamSynchronize(h->stream));
    cudaFree(h->d_rec_off);
    cudaFree(h->d_rec_comp);
    cudaFree(h->d_traces);
    h->d_rec_off = nullptr;
    h->d_rec_comp = nullptr;
    h->d_traces = nullptr;
    h->nrec = 0;
    if (n > 0) {
        CK(cudaMalloc(&h->d_rec_off, (size_t)n * sizeof(long long)));
        CK(cudaMalloc(&h->d_rec_comp, (size_t)n * sizeof(int)));
        CK(cudaMalloc(&h->d_traces, (size_t)n * h->p.nt * sizeof(double)));
        CK(cudaMemcpy(h->d_rec_off, off.data(), (size_t)n * sizeof(long long), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_rec_comp, comp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemset(h->d_traces, 0, (size_t)n * h->p.nt * sizeof(double)));
    }
    h->nrec = n;
    h->h_rec.assign(ijkc, ijkc + 4 * (size_t)n);
    h->graph_dirty = true;
    // the two-kernel step's velocity kernel samples the receivers itself when every one is a
    // velocity component on a cell its threads visit (1 <= i < nx, 1 <= j < ny, 1 <= k < nz)
    cudaFree(h->d_rcol);
    cudaFree(h->d_rent);
    h->d_rcol = nullptr;
    h->d_rent = nullptr;
    bool fuse = true;
    for (int r = 0; r < n; ++r) {
        const int i = ijkc[4 * r], j = ijkc[4 * r + 1], k = ijkc[4 * r + 2], c = ijkc[4 * r + 3];
        if (c > EWF_F_VZ || i < 1 || j < 1 || k < 1 || i >= h->p.nx || j >= h->p.ny || k >= h->p.nz) fuse = false;
    }
    h->rec_fuse = fuse;
    if (fuse && n > 0) {
        const size_t ncol = (size_t)h->p.nx * h->p.ny;
        std::vector<int> first(ncol, -1);
        std::vector<int4> ent((size_t)n);
        for (int r = n - 1; r >= 0; --r) {  // chained in list order
            const size_t col = (size_t)ijkc[4 * r] + (size_t)ijkc[4 * r + 1] * h->p.nx;
            ent[r] = make_int4(ijkc[4 * r + 2], ijkc[4 * r + 3], r, first[col]);
            first[col] = r;
        }
        CK(cudaMalloc(&h->d_rcol, ncol * sizeof(int)));
        CK(cudaMalloc(&h->d_rent, (size_t)n * sizeof(int4)));
        CK(cudaMemcpy(h->d_rcol, first.data(), ncol * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_rent, ent.data(), (size_t)n * sizeof(int4), cudaMemcpyHostToDevice));
    }
    return EWF_OK;
}

extern "C" int ewf_receiver_count(const ewf_handle *h, int32_t *n)
{
    if (!h || !n) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *n = h->nrec;
    return EWF_OK;
}

extern "C" int ewf_reset(ewf_handle *h)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    for (auto x : h->f_alloc) { int s = dev_zero(h, x); if (s) return s; }
    for (auto x : h->g_alloc) { int s = dev_zero(h, x); if (s) return s; }
    h->flip = 0;
    for (auto x : h->comp_alloc) { int s = dev_zero(h, x); if (s) return s; }
    if (h->d_traces) CK(cudaMemsetAsync(h->d_traces, 0, (size_t)h->nrec * h->p.nt * sizeof(double), h->stream));
    CK(cudaMemsetAsync(h->d_it, 0, 2 * sizeof(int), h->stream));
    if (h->d_wctl) {  // ticket and error flag; the generation keeps counting (stale done flags stay below it)
        CK(cudaMemsetAsync(&h->d_wctl->ticket, 0, sizeof(int), h->stream));
        CK(cudaMemsetAsync(&h->d_wctl->err, 0, sizeof(int), h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    h->it = 0;
    return EWF_OK;
}

// ------------------------------------------------------------------------------------------
// the time step
// ------------------------------------------------------------------------------------------
// A launch on the handle's stream; `pdl`: as a programmatic dependent of the stream's previous
// kernel (the kernel waits for it with griddepcontrol.wait before touching any state).
template <typename... P, typename... A>
static void launch_on(void (*kern)(P...), dim3 grid, dim3 block, cudaStream_t stream, bool pdl, A... args)
{
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// One step of the two-kernel form; `parity` = the step number's parity: the step counter of this
// step is d_it[parity], the next step's d_it[1 - parity].
template <typename T, int MODEL, int DAMP, bool KAHAN>
static void launch_step_t(const ewf_handle *h, const StepArgs<T> &a, cudaEvent_t *ev, int parity)
{
    const dim3 blk(TX, h->ty);
    const dim3 grd((h->p.nx + TX - 1) / TX, (h->p.ny + h->ty - 1) / h->ty, (h->p.nz + a.kchunk - 1) / a.kchunk);
    StressSrc ss = h->src_fuse;
    ss.stf = h->d_stf;
    ss.nstf = (int)h->nstf;
    int *const it_rd = h->d_it + parity, *const it_wr = h->d_it + (1 - parity);
    ss.it_ptr = it_rd;
    ss.order = h->p.src_order;
    RecFuse rf{};
    if (h->rec_fuse) {  // receivers sampled and the counter advanced by the velocity kernel
        rf.col_first = h->d_rcol;
        rf.ent = h->d_rent;
        rf.traces = h->d_traces;
        rf.trace_len = h->p.nt;
        rf.it_rd = it_rd;
        rf.it_wr = it_wr;
    }
    const bool pdl = h->pdl && !ev;  // kernels timed between events run as plain launches
    if (ev) cudaEventRecord(ev[0], h->stream);
    launch_on(k_stress<T, MODEL, DAMP>, grd, blk, h->stream, pdl, a, ss);
    if (ev) cudaEventRecord(ev[1], h->stream);
    if (h->nsrc > 0 && ss.nsrc == 0)
        launch_on(k_inject<T>, dim3(1), dim3(32), h->stream, pdl, a, (const SrcEntry *)h->d_src, h->nsrc,
                  (const double *)h->d_stf, (int)h->nstf, (const int *)it_rd, h->p.src_order);
    if (ev) cudaEventRecord(ev[2], h->stream);
    launch_on(k_velocity<T, MODEL, DAMP, KAHAN>, grd, blk, h->stream, pdl, a, rf);
    if (ev) cudaEventRecord(ev[3], h->stream);
    if (!h->rec_fuse)
        launch_on(k_record<T>, dim3(1), dim3(256), h->stream, pdl, a, (const long long *)h->d_rec_off,
                  (const int *)h->d_rec_comp, h->nrec, h->d_traces, (int)h->p.nt, (const int *)it_rd, it_wr);
    if (ev) cudaEventRecord(ev[4], h->stream);
}

// One time step.  `parity` selects the fused step's input buffer (0: f_alloc -> g_alloc).
typedef void (*step_fn)(const ewf_handle *, cudaEvent_t *, int parity);

template <typename T, int MODEL, int DAMP, bool KAHAN>
static void step_entry(const ewf_handle *h, cudaEvent_t *ev, int parity)
{
    const StepArgs<T> a = make_args<T>(h, 0);
    launch_step_t<T, MODEL, DAMP, KAHAN>(h, a, ev, parity);
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
static void fused_entry(const ewf_handle *h, cudaEvent_t *ev, int parity)
{
    FusedArgs<T> fa;
    memset(&fa, 0, sizeof(fa));
    fa.a = make_args<T>(h, parity);
    const StepArgs<T> out = make_args<T>(h, 1 - parity);
    for (int q = 0; q < 9; ++q) fa.o[q] = out.f[q];
    fa.src = h->d_src;
    fa.nsrc = h->nsrc;
    fa.stf = h->d_stf;
    fa.nstf = (int)h->nstf;
    fa.it_ptr = h->d_it;
    fa.order = h->p.src_order;
    if (ev) cudaEventRecord(ev[0], h->stream);
    const int rows = band_rows(h->onepass);
    bool staged = false;
    if constexpr (std::is_same<T, float>::value && !KAHAN) {
        if (h->onepass == EWF_ONEPASS_STAGED) {
            staged_launch<MODEL, DAMP>(fa, *h->splan, parity, h->hx, h->stream);
            staged = true;
        }
    }
    if (staged) {
    } else if (rows > 0) {
        band_launch<T, MODEL, DAMP, KAHAN>(fa, rows, band_grid(h->p.nx, h->p.ny, h->p.nz, rows, fa.a.kchunk), h->stream);
    } else {
        const dim3 blk(FX, FY);
        const dim3 grd((h->p.nx + FX - 1) / FX, (h->p.ny + FY - 1) / FY, (h->p.nz + fa.a.kchunk - 1) / fa.a.kchunk);
        k_step<T, MODEL, DAMP, KAHAN><<<grd, blk, 0, h->stream>>>(fa);
    }
    if (ev) {
        cudaEventRecord(ev[1], h->stream);
        cudaEventRecord(ev[2], h->stream);
        cudaEventRecord(ev[3], h->stream);
    }
    k_record<T><<<1, 256, 0, h->stream>>>(out, h->d_rec_off, h->d_rec_comp, h->nrec, h->d_traces, h->p.nt, h->d_it,
                                          h->d_it);
    if (ev) cudaEventRecord(ev[4], h->stream);
}

// The wavefront step: shape, done flags and the per-item grouping of the point sources for the
// current z-chunk (rebuilt when the chunk or the sources change; never during graph capture).
static WaveShape wave_shape_of(const ewf_handle *h, int lag)
{
    return wave_shape(h->p.nx, h->p.ny, h->p.nz, TX, TY, h->kchunk, lag);
}

static int wave_prepare(ewf_handle *h)
{
    if (!h->wave) return EWF_OK;
    const WaveShape w = wave_shape_of(h, 0);
    if (h->wave_key[0] == w.kslab && h->wave_key[1] == h->src_version && h->wave_key[2] == w.n) return EWF_OK;
    CK(cudaStreamSynchronize(h->stream));
    if (w.n > h->wdone_cap) {
        cudaFree(h->d_wdone);
        h->d_wdone = nullptr;
        h->wdone_cap = 0;
        CK(cudaMalloc(&h->d_wdone, (size_t)w.n * sizeof(int)));
        CK(cudaMemset(h->d_wdone, 0, (size_t)w.n * sizeof(int)));  // below every generation + 1
        h->wdone_cap = w.n;
    }
    // stable grouping by owner: entries of one item keep their order (k_inject's sum order)
    std::vector<int> off((size_t)w.n + 1, 0);
    std::vector<int> owner(h->h_src.size());
    for (size_t e = 0; e < h->h_src.size(); ++e) {
        const SrcEntry &q = h->h_src[e];
        owner[e] = wave_owner(w, TX, TY, q.i, q.j, q.k);
        off[(size_t)owner[e] + 1]++;
    }
    for (int i = 0; i < w.n; ++i) off[(size_t)i + 1] += off[(size_t)i];
    std::vector<SrcEntry> grouped(h->h_src.size());
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (size_t e = 0; e < h->h_src.size(); ++e) grouped[(size_t)fill[(size_t)owner[e]]++] = h->h_src[e];
    if (w.n + 1 > h->woff_cap) {
        cudaFree(h->d_woff);
        cudaFree(h->d_wsrc);
        h->d_woff = nullptr;
        h->d_wsrc = nullptr;
        h->woff_cap = 0;
        CK(cudaMalloc(&h->d_woff, (size_t)(w.n + 1) * sizeof(int)));
        CK(cudaMalloc(&h->d_wsrc, (size_t)MAXSRC * sizeof(SrcEntry)));
        h->woff_cap = w.n + 1;
    }
    CK(cudaMemcpy(h->d_woff, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (!grouped.empty())
        CK(cudaMemcpy(h->d_wsrc, grouped.data(), grouped.size() * sizeof(SrcEntry), cudaMemcpyHostToDevice));
    h->wave_key[0] = w.kslab;
    h->wave_key[1] = h->src_version;
    h->wave_key[2] = w.n;
    h->graph_dirty = true;
    return EWF_OK;
}

// reads and clears the wavefront step's error flag (after the stream has been synchronised)
static int wave_check(ewf_handle *h)
{
    if (!h->wave) return EWF_OK;
    WaveCtl c;
    CK(cudaMemcpy(&c, h->d_wctl, sizeof(c), cudaMemcpyDeviceToHost));
    if (c.err) {
        CK(cudaMemset(&h->d_wctl->err, 0, sizeof(int)));
        return ewf_fail(EWF_ERR_CUDA, "wavefront step: a dependency wait gave up; the state of this run is invalid");
    }
    return EWF_OK;
}

template <typename T, int MODEL, int DAMP, bool KAHAN>
static void wave_entry(const ewf_handle *h, cudaEvent_t *ev, int)
{
    const StepArgs<T> a = make_args<T>(h, 0);
    constexpr int MB = sizeof(T) == 4 ? 3 : 1;
    auto kern = k_wave<T, MODEL, DAMP, KAHAN, MB>;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WAVE_THREADS, 0);
    const WaveShape w0 = wave_shape_of(h, 0);
    int ctas = std::max(1, per_sm) * std::max(1, h->nsm);
    ctas = std::min(ctas, 2 * w0.n);
    WaveArgs wa;
    memset(&wa, 0, sizeof(wa));
    wa.w = wave_shape_of(h, w0.ntx + 1 + (int)((long long)ctas * h->wave_lag_pct / 100));
    wa.ctl = h->d_wctl;
    wa.done = h->d_wdone;
    wa.src_off = h->d_woff;
    wa.src = h->d_wsrc;
    wa.stf = h->d_stf;
    wa.nstf = (int)h->nstf;
    wa.it_ptr = h->d_it;
    wa.order = h->p.src_order;
    wa.hold = h->wave_hold;
    if (ev) cudaEventRecord(ev[0], h->stream);
    kern<<<ctas, WAVE_THREADS, 0, h->stream>>>(a, wa);
    if (ev) {
        cudaEventRecord(ev[1], h->stream);
        cudaEventRecord(ev[2], h->stream);
        cudaEventRecord(ev[3], h->stream);
    }
    k_record<T><<<1, 256, 0, h->stream>>>(a, h->d_rec_off, h->d_rec_comp, h->nrec, h->d_traces, h->p.nt, h->d_it,
                                          h->d_it);
    if (ev) cudaEventRecord(ev[4], h->stream);
}

// A step form: the host function that launches one step.
template <int FORM, typename T, int MODEL, int DAMP, bool KAHAN>
static step_fn entry()
{
    if constexpr (FORM == EWF_STEP_FUSED) return &fused_entry<T, MODEL, DAMP, KAHAN>;
    else if constexpr (FORM == EWF_STEP_WAVE) return &wave_entry<T, MODEL, DAMP, KAHAN>;
    else return &step_entry<T, MODEL, DAMP, KAHAN>;
}

// FORM: EWF_STEP_*; the one-pass form exists for models 0 and 1 with 1-D, 3-D or separable
// damping (validated), the others for every combination
template <int FORM>
static step_fn pick_step_t(const ewf_params &p)
{
    constexpr int F2 = FORM == EWF_STEP_FUSED ? EWF_STEP_SPLIT : FORM;  // forms built for every model
    const bool iso = p.model == EWF_MODEL_ISO;
    const bool w3 = p.damping == EWF_DAMP_W3D;
    if (p.damping == EWF_DAMP_PERCOMP) {
        switch (p.precision) {
        case EWF_PREC_F32: return entry<F2, float, MODEL_ISO, DAMP_PERCOMP, false>();
        case EWF_PREC_F32_KAHAN: return entry<F2, float, MODEL_ISO, DAMP_PERCOMP, true>();
        default: return entry<F2, double, MODEL_ISO, DAMP_PERCOMP, false>();
        }
    }
    if (p.model == EWF_MODEL_ISO_HET) {
        switch (p.precision) {
        case EWF_PREC_F32:
            return w3 ? entry<F2, float, MODEL_ISOHET, DAMP_W3D, false>() : entry<F2, float, MODEL_ISOHET, DAMP_SEP, false>();
        case EWF_PREC_F32_KAHAN:
            return w3 ? entry<F2, float, MODEL_ISOHET, DAMP_W3D, true>() : entry<F2, float, MODEL_ISOHET, DAMP_SEP, true>();
        default:
            return w3 ? entry<F2, double, MODEL_ISOHET, DAMP_W3D, false>() : entry<F2, double, MODEL_ISOHET, DAMP_SEP, false>();
        }
    }
    switch (p.precision) {
    case EWF_PREC_F32:
        if (iso) return entry<FORM, float, MODEL_ISO, DAMP_PML1D, false>();
        return w3 ? entry<FORM, float, MODEL_ORTHO, DAMP_W3D, false>() : entry<FORM, float, MODEL_ORTHO, DAMP_SEP, false>();
    case EWF_PREC_F32_KAHAN:
        if (iso) return entry<FORM, float, MODEL_ISO, DAMP_PML1D, true>();
        return w3 ? entry<FORM, float, MODEL_ORTHO, DAMP_W3D, true>() : entry<FORM, float, MODEL_ORTHO, DAMP_SEP, true>();
    default:
        if (iso) return entry<FORM, double, MODEL_ISO, DAMP_PML1D, false>();
        return w3 ? entry<FORM, double, MODEL_ORTHO, DAMP_W3D, false>() : entry<FORM, double, MODEL_ORTHO, DAMP_SEP, false>();
    }
}

// Can the band kernel of the one-pass step run with `rows` rows per CTA on this handle's grid
// (built for the element type, at most BAND_MAX_CTAS CTAs per band, a cluster fits the device)?
template <typename T, int MODEL, int DAMP, bool KAHAN>
static bool band_fits_t(const ewf_handle *h, int rows)
{
    if (!band_rows_built<T>(rows)) return false;
    int n = 0;
    const cudaError_t e = band_clusters<T, MODEL, DAMP, KAHAN>(rows, band_grid(h->p.nx, h->p.ny, h->p.nz, rows, h->kchunk), &n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return n >= 1;
}

// Can the staged kernel run on this handle (FP32 without compensation, models 0 and 1 with the
// one-pass form's dampings, shared memory on this device, tensor maps of its allocations)?
// Encodes the maps on first use.
static bool staged_fits(ewf_handle *h)
{
    const ewf_params &p = h->p;
    if (!h->fused || p.precision != EWF_PREC_F32 || p.damping == EWF_DAMP_PERCOMP || p.model == EWF_MODEL_ISO_HET) return false;
    const bool iso = p.model == EWF_MODEL_ISO, w3 = p.damping == EWF_DAMP_W3D;
    const bool ready = iso ? staged_ready<MODEL_ISO, DAMP_PML1D>()
                           : (w3 ? staged_ready<MODEL_ORTHO, DAMP_W3D>() : staged_ready<MODEL_ORTHO, DAMP_SEP>());
    if (!ready) return false;
    if (!h->splan) {
        h->splan = new (std::nothrow) StagedPlan();
        if (!h->splan) return false;
        static const int slots[9] = {0, 1, 2, 3, 4, 5, 6, 7, 8};
        staged_encode(*h->splan, h->f_alloc, h->g_alloc, h->m_alloc, h->w3_alloc, iso ? 2 : 9, slots, !iso && w3, !iso,
                      h->sx, p.ny, p.nz);
    }
    return h->splan->ok;
}

static bool band_fits(const ewf_handle *h, int rows)
{
    const ewf_params &p = h->p;
    if (!h->fused || p.damping == EWF_DAMP_PERCOMP || p.model == EWF_MODEL_ISO_HET) return false;
    const bool iso = p.model == EWF_MODEL_ISO, w3 = p.damping == EWF_DAMP_W3D;
    switch (p.precision) {
    case EWF_PREC_F32:
        if (iso) return band_fits_t<float, MODEL_ISO, DAMP_PML1D, false>(h, rows);
        return w3 ? band_fits_t<float, MODEL_ORTHO, DAMP_W3D, false>(h, rows) : band_fits_t<float, MODEL_ORTHO, DAMP_SEP, false>(h, rows);
    case EWF_PREC_F32_KAHAN:
        if (iso) return band_fits_t<float, MODEL_ISO, DAMP_PML1D, true>(h, rows);
        return w3 ? band_fits_t<float, MODEL_ORTHO, DAMP_W3D, true>(h, rows) : band_fits_t<float, MODEL_ORTHO, DAMP_SEP, true>(h, rows);
    default:
        if (iso) return band_fits_t<double, MODEL_ISO, DAMP_PML1D, false>(h, rows);
        return w3 ? band_fits_t<double, MODEL_ORTHO, DAMP_W3D, false>(h, rows) : band_fits_t<double, MODEL_ORTHO, DAMP_SEP, false>(h, rows);
    }
}

static step_fn pick_step(const ewf_handle *h)
{
    if (h->fused) return pick_step_t<EWF_STEP_FUSED>(h->p);
    if (h->wave) return pick_step_t<EWF_STEP_WAVE>(h->p);
    return pick_step_t<EWF_STEP_SPLIT>(h->p);
}

// everything a step form needs built before its first launch (never during capture)
static int step_prepare(ewf_handle *h)
{
    return wave_prepare(h);
}
static int step_check(ewf_handle *h)
{
    if (h->fused && h->onepass == EWF_ONEPASS_STAGED && staged_take_error())
        return ewf_fail(EWF_ERR_CUDA, "staged one-pass step: a wait for a plane stage gave up; the state of this run is invalid");
    return wave_check(h);
}

static int inputs_ready(const ewf_handle *h)
{
    for (int q = 0; q < n_materials(h->p.model); ++q)
        if (slot_used(h->p.model, q) && !h->m_set[q]) return ewf_fail(EWF_ERR_STATE, "material slot %d not set", q);
    if (h->p.damping == EWF_DAMP_W3D) {
        if (!h->w_set[3]) return ewf_fail(EWF_ERR_STATE, "3-D weights not set");
    } else if (h->p.damping == EWF_DAMP_PERCOMP) {
        for (int q = 4; q < 10; ++q)
            if (!h->w_set[q]) return ewf_fail(EWF_ERR_STATE, "per-component weights %d not set", q - 4);
    } else {
        for (int q = 0; q < 3; ++q)
            if (!h->w_set[q]) return ewf_fail(EWF_ERR_STATE, "damping profile %d not set", q);
    }
    if (h->nsrc > 0 && !h->d_stf) return ewf_fail(EWF_ERR_STATE, "sources set but no source time function");
    return EWF_OK;
}

// The two-kernel step keeps its step counter in two alternating device locations (d_it[it & 1]).
static bool split_form(const ewf_handle *h) { return !h->fused && !h->wave; }

static int build_graph(ewf_handle *h, step_fn fn)
{
    if (h->gexec) {
        cudaGraphExecDestroy(h->gexec);
        h->gexec = nullptr;
    }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < h->gsteps; ++s) fn(h, nullptr, (h->dbuf || split_form(h)) ? (s & 1) : 0);
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return ewf_fail(EWF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    const cudaError_t ie = cudaGraphInstantiate(&h->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        h->gexec = nullptr;
        return ewf_fail(EWF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
    }
    h->graph_dirty = false;
    return EWF_OK;
}

extern "C" int ewf_run(ewf_handle *h, int32_t nsteps)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (nsteps < 0) return ewf_fail(EWF_ERR_ARG, "nsteps < 0");
    int st = inputs_ready(h);
    if (st) return st;
    if (h->it + nsteps > h->p.nt)
        return ewf_fail(EWF_ERR_ARG, "step %d + %d exceeds nt = %d", h->it, nsteps, h->p.nt);
    if (h->nsrc > 0 && (size_t)(h->it + nsteps) > h->nstf)
        return ewf_fail(EWF_ERR_ARG, "source time function has %zu samples, need %d", h->nstf, h->it + nsteps);
    if ((st = step_prepare(h))) return st;
    const step_fn fn = pick_step(h);
    // steps alternate a parity: the one-pass form's buffers, the two-kernel step's counter; the
    // graph starts at parity 0
    const bool alt = h->dbuf || split_form(h);
    int parity = h->dbuf ? h->flip : (split_form(h) ? (h->it & 1) : 0);
    const bool use_graph = h->gsteps > 0 && nsteps >= h->gsteps + parity;
    bool graph = use_graph;
    if (graph && (h->graph_dirty || !h->gexec)) {
        st = build_graph(h, fn);
        if (st && h->pdl) {  // a driver that cannot capture dependent launches: plain ones
            cudaGetLastError();
            h->pdl = false;
            st = build_graph(h, fn);
        }
        if (st) return st;
    }
    CK(cudaEventRecord(h->ev0, h->stream));
    int done = 0;
    if (graph && parity) {  // the graph starts from parity 0: one direct step first
        fn(h, nullptr, parity);
        parity = 0;
        ++done;
    }
    if (graph) {
        for (; done + h->gsteps <= nsteps; done += h->gsteps) {
            CK(cudaGraphLaunch(h->gexec, h->stream));
            if (h->p.nout > 0 && ((h->it + done) / h->p.nout) != ((h->it + done + h->gsteps) / h->p.nout)) {
                printf("it=%05d > ", h->it + done + h->gsteps);
                fflush(stdout);
            }
        }
    }
    for (; done < nsteps; ++done) {
        fn(h, nullptr, parity);
        if (alt) parity ^= 1;
    }
    h->flip = h->dbuf ? parity : 0;
    CK(cudaGetLastError());
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaEventElapsedTime(&h->last_ms, h->ev0, h->ev1));
    h->it += nsteps;
    if ((st = step_check(h))) return st;
    if (h->p.check_finite && h->nrec > 0 && nsteps > 0) {
        // only the samples of this call: columns [it - nsteps, it) of the nrec x nt traces
        const int t0 = h->it - nsteps;
        std::vector<double> tr((size_t)h->nrec * nsteps);
        CK(cudaMemcpy2D(tr.data(), (size_t)nsteps * sizeof(double), h->d_traces + t0, (size_t)h->p.nt * sizeof(double),
                        (size_t)nsteps * sizeof(double), (size_t)h->nrec, cudaMemcpyDeviceToHost));
        for (int r = 0; r < h->nrec; ++r)
            for (int t = 0; t < nsteps; ++t)
                if (!std::isfinite(tr[(size_t)r * nsteps + t]))
                    return ewf_fail(EWF_ERR_NONFINITE, "receiver %d has a non-finite sample at step %d", r, t0 + t);
    }
    return EWF_OK;
}

extern "C" int ewf_time_kernels(ewf_handle *h, int32_t nsteps, double out_ms[4])
{
    if (!h || !out_ms || nsteps < 1) return ewf_fail(EWF_ERR_ARG, "bad argument");
    int st = inputs_ready(h);
    if (st) return st;
    if (h->it + nsteps > h->p.nt) return ewf_fail(EWF_ERR_ARG, "step %d + %d exceeds nt = %d", h->it, nsteps, h->p.nt);
    if (h->nsrc > 0 && (size_t)(h->it + nsteps) > h->nstf) return ewf_fail(EWF_ERR_ARG, "source time function too short");
    if ((st = step_prepare(h))) return st;
    const step_fn fn = pick_step(h);
    cudaEvent_t ev[5] = {};
    for (auto &e : ev) CK(cudaEventCreate(&e));
    double acc[4] = {0, 0, 0, 0};
    int err = EWF_OK;
    for (int s = 0; s < nsteps && !err; ++s) {
        fn(h, ev, h->dbuf ? h->flip : ((h->it + s) & 1));
        if (h->dbuf) h->flip ^= 1;
        if (cudaEventSynchronize(ev[4]) != cudaSuccess) { err = ewf_fail(EWF_ERR_CUDA, "kernel timing: %s", cudaGetErrorString(cudaGetLastError())); break; }
        for (int q = 0; q < 4; ++q) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[q], ev[q + 1]);
            acc[q] += ms;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (err) return err;
    CK(cudaGetLastError());
    h->it += nsteps;
    if ((st = step_check(h))) return st;
    for (int q = 0; q < 4; ++q) out_ms[q] = acc[q] / nsteps;
    return EWF_OK;
}

// Device time of `steps` steps from a reset state (one untimed step first); -1 when the current
// settings cannot run.
static int time_setting(ewf_handle *h, int steps, float *ms)
{
    int st = ewf_reset(h);
    if (st) return st;
    if (step_prepare(h)) {
        *ms = -1.f;
        return EWF_OK;
    }
    const step_fn fn = pick_step(h);
    fn(h, nullptr, h->flip);  // warm (step 0 after the reset)
    if (h->dbuf) h->flip ^= 1;
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int s = 0; s < steps; ++s) {
        fn(h, nullptr, h->dbuf ? h->flip : ((s + 1) & 1));
        if (h->dbuf) h->flip ^= 1;
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if ((st = step_check(h))) return st;
    CK(cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return EWF_OK;
}

extern "C" int ewf_autotune(ewf_handle *h, int32_t nsteps, int32_t *kchunk)
{
    if (!h || nsteps < 1) return ewf_fail(EWF_ERR_ARG, "bad argument");
    int st = inputs_ready(h);
    if (st) return st;
    static const int cand[] = {4, 6, 8, 12, 16, 24, 32, 48, 64};
    const int steps = std::min(nsteps, h->p.nt - 1);
    if (steps < 1) return ewf_fail(EWF_ERR_ARG, "nt too small to tune");
    if (h->nsrc > 0 && h->nstf < (size_t)steps + 1) return ewf_fail(EWF_ERR_STATE, "source time function too short");
    float best = 1e30f;
    if (h->fused) {
        // one-pass step: kernel (0: tile kernel, 4 / 8: band kernel rows per CTA) x z-chunk (each
        // chunk recomputes two extra stress planes, so longer chunks than the other forms')
        static const int bcand[] = {8, 16, 24, 32, 48, 64, 96, 128};
        static const int kern_cand[] = {EWF_ONEPASS_TILE, EWF_ONEPASS_BAND4, EWF_ONEPASS_BAND8, EWF_ONEPASS_STAGED};
        int best_kern = h->onepass, best_kc = h->kchunk;
        for (int kern : kern_cand) {
            if (band_rows(kern) > 0 && !band_fits(h, band_rows(kern))) continue;
            if (kern == EWF_ONEPASS_STAGED && !staged_fits(h)) continue;
            for (int kc : bcand) {
                if (kc > h->p.nz && kc != bcand[0]) continue;
                h->onepass = kern;
                h->kchunk = std::max(4, std::min(kc, h->p.nz));
                float ms = 0.f;
                if ((st = time_setting(h, steps, &ms))) return st;
                if (ms >= 0.f && ms < best) {
                    best = ms;
                    best_kern = kern;
                    best_kc = h->kchunk;
                }
            }
        }
        h->onepass = best_kern;
        h->kchunk = best_kc;
        h->graph_dirty = true;
        if (kchunk) *kchunk = best_kc;
        return ewf_reset(h);
    }
    int best_k = h->kchunk, best_lag = h->wave_lag_pct, best_ty = h->ty;
    // wavefront step: slabs of 4..16 planes x lag (100000: every stress item before the first velocity item)
    static const int lag_pct[] = {50, 100, 200, 100000};
    const int nvar = h->wave ? 4 : 1;
    // two-kernel step: z-chunk x tile height (rows of 32 columns per CTA)
    const bool split = !h->wave && !h->fused;
    static const int ty_cand[] = {4, 8, 16};
    for (int ty : ty_cand) {
        if (!split && ty != h->ty) continue;
        if (ty > (h->esz == 4 ? SPLIT_MAX_TY : TY)) continue;
        for (int kc : cand) {
            if (kc > h->p.nz && kc != cand[0]) continue;
            if (h->wave && kc > 16) continue;
            for (int vi = 0; vi < nvar; ++vi) {
                h->kchunk = std::max(4, std::min(kc, h->p.nz));
                h->ty = ty;
                if (h->wave) {
                    h->wave_lag_pct = lag_pct[vi];
                    h->graph_dirty = true;
                }
                float ms = 0.f;
                if ((st = time_setting(h, steps, &ms))) return st;
                if (ms >= 0.f && ms < best) {
                    best = ms;
                    best_k = h->kchunk;
                    best_lag = h->wave_lag_pct;
                    best_ty = h->ty;
                }
            }
        }
    }
    h->kchunk = best_k;
    h->ty = best_ty;
    h->wave_lag_pct = best_lag;
    if (split) {  // then the velocity kernel's L2 prefetch distance at that setting
        int best_pf = 0;
        h->l2pf = 0;
        float base = 0.f;
        if ((st = time_setting(h, steps, &base))) return st;
        best = base;
        static const int pf_cand[] = {2, 3, 4};
        for (int pf : pf_cand) {
            h->l2pf = pf;
            float ms = 0.f;
            if ((st = time_setting(h, steps, &ms))) return st;
            if (ms >= 0.f && ms < best) {
                best = ms;
                best_pf = pf;
            }
        }
        h->l2pf = best_pf;
    }
    h->graph_dirty = true;
    if (kchunk) *kchunk = best_k;
    return ewf_reset(h);
}

extern "C" int ewf_set_tile(ewf_handle *h, int32_t tile_y)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (h->wave || h->fused) return ewf_fail(EWF_ERR_STATE, "the tile height applies to the two-kernel step");
    const int mx = h->esz == 4 ? SPLIT_MAX_TY : TY;
    if (tile_y < 1 || tile_y > mx || (tile_y & (tile_y - 1)))
        return ewf_fail(EWF_ERR_ARG, "tile_y must be a power of two in [1, %d] (got %d)", mx, tile_y);
    h->ty = tile_y;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_set_l2_prefetch(ewf_handle *h, int32_t planes)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (planes < 0 || planes > 8) return ewf_fail(EWF_ERR_ARG, "planes must be in [0, 8] (got %d)", planes);
    h->l2pf = planes;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_get_l2_prefetch(const ewf_handle *h, int32_t *planes)
{
    if (!h || !planes) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *planes = h->l2pf;
    return EWF_OK;
}

extern "C" int ewf_set_dependent_launch(ewf_handle *h, int32_t on)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    h->pdl = on != 0;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_get_dependent_launch(const ewf_handle *h, int32_t *on)
{
    if (!h || !on) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *on = h->pdl ? 1 : 0;
    return EWF_OK;
}

extern "C" int ewf_set_onepass(ewf_handle *h, int32_t kernel)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (!h->fused) return ewf_fail(EWF_ERR_STATE, "the one-pass kernel applies to the one-pass step");
    if (kernel < EWF_ONEPASS_TILE || kernel > EWF_ONEPASS_STAGED) return ewf_fail(EWF_ERR_ARG, "unknown one-pass kernel %d", kernel);
    const int rows = band_rows(kernel);
    if (rows > 0 && !band_fits(h, rows))
        return ewf_fail(EWF_ERR_UNSUPPORTED, "band kernel with %d rows: not built for this precision, more than %d CTAs of "
                        "%d columns per band, or no cluster of that size fits the device", rows, BAND_MAX_CTAS, BX);
    if (kernel == EWF_ONEPASS_STAGED) {
        cudaSetDevice(h->device);
        if (!staged_fits(h))
            return ewf_fail(EWF_ERR_UNSUPPORTED, "staged kernel: built for FP32 without compensation and models 0 and 1; "
                            "needs ~220 KB of shared memory per block and the driver's tensor-map encoder");
    }
    h->onepass = kernel;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_staged_test_hold(int32_t plane, int32_t polls)
{
    if (staged_test_hold(plane, polls)) return ewf_fail(EWF_ERR_CUDA, "staged test hook: %s", cudaGetErrorString(cudaGetLastError()));
    return EWF_OK;
}

extern "C" int ewf_get_onepass(const ewf_handle *h, int32_t *kernel)
{
    if (!h || !kernel) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *kernel = h->onepass;
    return EWF_OK;
}

extern "C" int ewf_get_tile(const ewf_handle *h, int32_t *tile_y)
{
    if (!h || !tile_y) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *tile_y = h->ty;
    return EWF_OK;
}

extern "C" int ewf_set_wave(ewf_handle *h, int32_t lag_pct)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (!h->wave) return ewf_fail(EWF_ERR_STATE, "not a wavefront-step handle");
    if (lag_pct < 1 || lag_pct > 100000) return ewf_fail(EWF_ERR_ARG, "lag_pct must be in [1, 100000] (got %d)", lag_pct);
    h->wave_lag_pct = lag_pct;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_wave_hold(ewf_handle *h, int32_t item)
{
    if (!h) return ewf_fail(EWF_ERR_ARG, "NULL handle");
    if (!h->wave) return ewf_fail(EWF_ERR_STATE, "not a wavefront-step handle");
    if (item < -1) return ewf_fail(EWF_ERR_ARG, "item must be >= -1");
    h->wave_hold = item;
    h->graph_dirty = true;
    return EWF_OK;
}

extern "C" int ewf_get_wave(const ewf_handle *h, int32_t *lag_pct)
{
    if (!h || !lag_pct) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    if (!h->wave) return ewf_fail(EWF_ERR_STATE, "not a wavefront-step handle");
    *lag_pct = h->wave_lag_pct;
    return EWF_OK;
}

extern "C" int ewf_launches_per_step(const ewf_handle *h, int32_t *n)
{
    if (!h || !n) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *n = (h->fused || h->wave) ? 2 : 2 + (h->nsrc > 0 && h->src_fuse.nsrc == 0 ? 1 : 0) + (h->rec_fuse ? 0 : 1);
    return EWF_OK;
}

extern "C" int ewf_get_step(const ewf_handle *h, int32_t *it)
{
    if (!h || !it) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *it = h->it;
    return EWF_OK;
}

extern "C" int ewf_last_run_ms(const ewf_handle *h, double *ms)
{
    if (!h || !ms) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *ms = h->last_ms;
    return EWF_OK;
}

extern "C" int ewf_get_seismograms(ewf_handle *h, double *out, size_t n)
{
    if (!h || (!out && n)) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    const size_t need = (size_t)h->nrec * h->p.nt;
    if (n != need) return ewf_fail(EWF_ERR_ARG, "%zu samples given, %zu expected (n_rec x nt)", n, need);
    if (need) CK(cudaMemcpyAsync(out, h->d_traces, need * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return EWF_OK;
}

// ------------------------------------------------------------------------------------------
// checkpoint / restore: header, 9 state fields (+3 compensation), traces -- reference layout
// ------------------------------------------------------------------------------------------
struct CkptHeader {
    char magic[8];
    int32_t version, nx, ny, nz, nt, model, precision, damping, it, nrec, ncomp, pad;
};

extern "C" int ewf_checkpoint(ewf_handle *h, const char *path)
{
    if (!h || !path) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    FILE *fp = fopen(path, "wb");
    if (!fp) return ewf_fail(EWF_ERR_IO, "cannot open %s for writing", path);
    CkptHeader hd;
    memset(&hd, 0, sizeof(hd));
    memcpy(hd.magic, "EWFCKPT1", 8);
    hd.version = 1; hd.nx = h->p.nx; hd.ny = h->p.ny; hd.nz = h->p.nz; hd.nt = h->p.nt;
    hd.model = h->p.model; hd.precision = h->p.precision; hd.damping = h->p.damping;
    hd.it = h->it; hd.nrec = h->nrec; hd.ncomp = h->comp_alloc[0] ? 3 : 0;
    int st = EWF_OK;
    if (fwrite(&hd, sizeof(hd), 1, fp) != 1) st = ewf_fail(EWF_ERR_IO, "write %s", path);
    std::vector<char> buf;
    for (int q = 0; q < 9 + hd.ncomp && !st; ++q) {
        const int id = q < 9 ? q : q - 9;
        const size_t n = ewf_field_size(h, id);
        buf.resize(n * h->esz);
        if (q < 9) {
            st = ewf_get_field(h, id, buf.data(), n, (int)h->esz);
        } else {
            // compensation arrays share Vx/Vy/Vz extents; unpack directly
            int ex, ey, ez;
            ewf_field_extent(h->p, id, &ex, &ey, &ez);
            k_unpack<float, float><<<pack_blocks(n), 256, 0, h->stream>>>((float *)h->d_stage,
                (const float *)boxptr(h, h->comp_alloc[id]), ex, ey, ez, h->sx, h->sy);
            if (cudaMemcpyAsync(buf.data(), h->d_stage, n * 4, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
                cudaStreamSynchronize(h->stream) != cudaSuccess)
                st = ewf_fail(EWF_ERR_CUDA, "checkpoint: compensation copy failed");
        }
        if (!st && fwrite(buf.data(), 1, buf.size(), fp) != buf.size()) st = ewf_fail(EWF_ERR_IO, "write %s", path);
    }
    if (!st && h->nrec) {
        std::vector<double> tr((size_t)h->nrec * h->p.nt);
        st = ewf_get_seismograms(h, tr.data(), tr.size());
        if (!st && fwrite(tr.data(), sizeof(double), tr.size(), fp) != tr.size()) st = ewf_fail(EWF_ERR_IO, "write %s", path);
    }
    if (fclose(fp) != 0 && !st) st = ewf_fail(EWF_ERR_IO, "close %s", path);
    return st;
}

extern "C" int ewf_restore(ewf_handle *h, const char *path)
{
    if (!h || !path) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    FILE *fp = fopen(path, "rb");
    if (!fp) return ewf_fail(EWF_ERR_IO, "cannot open %s", path);
    CkptHeader hd;
    int st = EWF_OK;
    if (fread(&hd, sizeof(hd), 1, fp) != 1 || memcmp(hd.magic, "EWFCKPT1", 8) != 0) st = ewf_fail(EWF_ERR_IO, "%s is not a checkpoint", path);
    if (!st && (hd.nx != h->p.nx || hd.ny != h->p.ny || hd.nz != h->p.nz || hd.nt != h->p.nt || hd.model != h->p.model ||
                hd.precision != h->p.precision || hd.nrec != h->nrec))
        st = ewf_fail(EWF_ERR_ARG, "checkpoint %s does not match this handle (grid/model/precision/receivers)", path);
    std::vector<char> buf;
    for (int q = 0; q < 9 + hd.ncomp && !st; ++q) {
        const int id = q < 9 ? q : q - 9;
        const size_t n = ewf_field_size(h, id);
        buf.resize(n * h->esz);
        if (fread(buf.data(), 1, buf.size(), fp) != buf.size()) { st = ewf_fail(EWF_ERR_IO, "short read %s", path); break; }
        if (q < 9) {
            st = ewf_set_field(h, id, buf.data(), n, (int)h->esz);
        } else if (h->comp_alloc[id]) {
            int ex, ey, ez;
            ewf_field_extent(h->p, id, &ex, &ey, &ez);
            if (cudaMemcpyAsync(h->d_stage, buf.data(), n * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
                st = ewf_fail(EWF_ERR_CUDA, "restore: compensation copy failed");
            k_pack<float, float><<<pack_blocks(n), 256, 0, h->stream>>>((float *)boxptr(h, h->comp_alloc[id]),
                (const float *)h->d_stage, ex, ey, ez, h->sx, h->sy);
            if (cudaStreamSynchronize(h->stream) != cudaSuccess) st = ewf_fail(EWF_ERR_CUDA, "restore: sync failed");
        }
    }
    if (!st && h->nrec) {
        std::vector<double> tr((size_t)h->nrec * h->p.nt);
        if (fread(tr.data(), sizeof(double), tr.size(), fp) != tr.size()) st = ewf_fail(EWF_ERR_IO, "short read %s", path);
        else if (cudaMemcpy(h->d_traces, tr.data(), tr.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
            st = ewf_fail(EWF_ERR_CUDA, "restore: trace copy failed");
    }
    fclose(fp);
    if (!st) {
        const int it2[2] = {hd.it, hd.it};  // both counter locations (the two-kernel step reads d_it[it & 1])
        if (cudaMemcpy(h->d_it, it2, sizeof(it2), cudaMemcpyHostToDevice) != cudaSuccess) return ewf_fail(EWF_ERR_CUDA, "restore: step copy");
        const int it = hd.it;
        h->it = it;
    }
    return st;
}

// ------------------------------------------------------------------------------------------
// Layout conversion without device allocation (ewf_pack_field_noalloc).  The staging scratch
// that ewf_set_field takes from its handle is, here, a fixed array compiled into the library;
// host code only ever passes the array's device address, looked up once per device.
// ------------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_pack_scratch[EWF_NOALLOC_SCRATCH_BYTES];

// Device address of g_pack_scratch on the current device.  Looked up on every call (a host-side
// query, no stream work), so a context that was torn down and created again -- where the
// library's device code may sit at a new address -- never sees a stale address.
static int pack_scratch_address(void **out)
{
    int dev = -1;
    CK(cudaGetDevice(&dev));
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_pack_scratch);
    if (e != cudaSuccess || !p)
        return ewf_fail(EWF_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d: %s", dev, cudaGetErrorString(e));
    *out = p;
    return EWF_OK;
}

// The allocation that contains device address p (base and size), through the driver's
// cuMemGetAddressRange, reached by the runtime's entry-point query so the library needs no
// link against the driver library.  Returns false where the driver does not know p.
static bool device_allocation_range(const void *p, unsigned long long *base, size_t *size)
{
    typedef int (*range_fn)(unsigned long long *, size_t *, unsigned long long);
    static range_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (range_fn)f;
        cudaGetLastError();
    });
    return fn && fn(base, size, (unsigned long long)(uintptr_t)p) == 0;
}

extern "C" int ewf_pack_field_noalloc(void *dst, int32_t dst_dtype_bytes, int32_t sx, int64_t sy, const void *host,
                                      int32_t host_dtype_bytes, int32_t ex, int32_t ey, int32_t ez, void *stream)
{
    if (!dst || !host) return ewf_fail(EWF_ERR_ARG, "NULL pointer");
    if ((dst_dtype_bytes != 4 && dst_dtype_bytes != 8) || (host_dtype_bytes != 4 && host_dtype_bytes != 8))
        return ewf_fail(EWF_ERR_ARG, "dtype bytes must be 4 or 8");
    if (ex < 1 || ey < 1 || ez < 1) return ewf_fail(EWF_ERR_ARG, "extent %dx%dx%d", ex, ey, ez);
    if (sx < ex || sy < (int64_t)sx * ey || sy > (int64_t(1) << 40))
        return ewf_fail(EWF_ERR_ARG, "pitches sx=%d sy=%lld do not hold %dx%d rows", sx, (long long)sy, ex, ey);
    const size_t n = (size_t)ex * ey * ez;
    const size_t bytes = n * (size_t)host_dtype_bytes;
    if (bytes > EWF_NOALLOC_SCRATCH_BYTES)
        return ewf_fail(EWF_ERR_ARG, "array of %zu bytes exceeds the %u-byte no-allocation scratch", bytes,
                        (unsigned)EWF_NOALLOC_SCRATCH_BYTES);
    if ((uintptr_t)dst % (uintptr_t)dst_dtype_bytes != 0)
        return ewf_fail(EWF_ERR_ARG, "dst %p is not aligned to its %d-byte elements", dst, dst_dtype_bytes);
    // dst must be device memory of the current device (or managed memory), and the last element
    // the conversion writes must lie inside dst's allocation: checked here so that a wrong
    // pointer becomes EWF_ERR_ARG instead of a kernel's out-of-range access
    int dev = -1;
    CK(cudaGetDevice(&dev));
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, dst) != cudaSuccess) {
        cudaGetLastError();
        return ewf_fail(EWF_ERR_ARG, "dst %p is not memory the CUDA runtime knows", dst);
    }
    if (pa.type == cudaMemoryTypeDevice ? pa.device != dev : pa.type != cudaMemoryTypeManaged)
        return ewf_fail(EWF_ERR_ARG, "dst %p is not device memory of device %d or managed memory", dst, dev);
    const unsigned long long last = (unsigned long long)(uintptr_t)dst +
        ((unsigned long long)(ex - 1) + (unsigned long long)(ey - 1) * (unsigned)sx + (unsigned long long)(ez - 1) * sy +
         1ull) * (unsigned)dst_dtype_bytes;
    unsigned long long abase = 0;
    size_t asize = 0;
    if (!device_allocation_range(dst, &abase, &asize))
        return ewf_fail(EWF_ERR_ARG, "dst %p: its allocation range is unknown to the driver", dst);
    if (last > abase + asize)
        return ewf_fail(EWF_ERR_ARG, "dst %p: the %dx%dx%d extent with pitches %d, %lld ends %llu bytes past its allocation",
                        dst, ex, ey, ez, sx, (long long)sy, last - (abase + asize));
    void *scratch = nullptr;
    const int st = pack_scratch_address(&scratch);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(scratch, host, bytes, cudaMemcpyHostToDevice, s));
    const unsigned nb = pack_blocks(n);
    if (dst_dtype_bytes == 4) {
        if (host_dtype_bytes == 4) k_pack<float, float><<<nb, 256, 0, s>>>((float *)dst, (const float *)scratch, ex, ey, ez, sx, sy);
        else k_pack<float, double><<<nb, 256, 0, s>>>((float *)dst, (const double *)scratch, ex, ey, ez, sx, sy);
    } else {
        if (host_dtype_bytes == 4) k_pack<double, float><<<nb, 256, 0, s>>>((double *)dst, (const float *)scratch, ex, ey, ez, sx, sy);
        else k_pack<double, double><<<nb, 256, 0, s>>>((double *)dst, (const double *)scratch, ex, ey, ez, sx, sy);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    return EWF_OK;
}
