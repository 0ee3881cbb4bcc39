// ewfd_batch.cu -- the batched solver (ewf_batch_*) and the z-chunk autotuner.
//
// The reference runs one model and one source per process (README.md:86-102; one scenario
// directory per run).  A batch holds several problems (models, possibly of different sizes and
// model families) with several right-hand sides each, advanced together: per time step one
// persistent stress launch and one velocity launch per model family, one injection launch and
// one receiver launch for everything -- captured in a CUDA graph.
#include "ewfd.h"
#include "ewfd_internal.h"
#include "ewfd_batch.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

using namespace ewf;

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return ewf_fail(e_ == cudaErrorMemoryAllocation ? EWF_ERR_NOMEM : EWF_ERR_CUDA,          \
                            "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);     \
    } while (0)

namespace {

struct Prob {
    ewf_params p;
    int R = 1;
    int sx = 0;             // materials / damping box
    long long sy = 0;
    size_t box = 0;
    long long base_off = 0;
    int sxs = 0;            // state box pitches (the material box's) and size of the R boxes
    long long sys = 0;
    size_t sbox = 0;
    long long sbase_off = 0;
    void *state[9] = {};
    void *mats[12] = {};
    void *w1[3] = {};
    void *w3 = nullptr;
    bool m_set[12] = {};
    bool w_set[4] = {};
    int kchunk = 16;
    bool fdiv = false;                      // div_spacing verified for dx, dy, dz
    std::vector<int32_t> rec;               // n x (i,j,k,comp)
    std::vector<std::vector<BatchSrc>> src;  // per RHS
    std::vector<double> stf;
};

struct Family {
    int model, damping;           // single-RHS problems of one (model, damping) share a launch
    std::vector<int> probs;       // problem indices
    BatchProb<float> *d_probs = nullptr;
    int *d_item0 = nullptr;
    int nitems = 0;
    int grid_stress = 0, grid_vel = 0;
    int ty = TY;                  // CTA tile height of the family's launches
};

float *bptr(const Prob &q, void *alloc) { return alloc ? (float *)alloc + q.base_off : nullptr; }
float *sptr(const Prob &q, void *alloc) { return alloc ? (float *)alloc + q.sbase_off : nullptr; }

}  // namespace

struct ewf_batch {
    int device = 0;
    int nt = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<Prob> probs;
    std::vector<Family> fams;
    BatchProb<float> *d_all = nullptr;  // every problem, indexed by problem id
    std::vector<BatchProb<float>> h_all;  // host copy of d_all
    std::vector<int> mr;                  // problems with several RHS: launched on their own
    int nrhs_total = 0;
    // sources
    BatchSrc *d_src = nullptr;
    int *d_src_start = nullptr;
    int ngroups = 0;
    double *d_stf = nullptr;
    int *d_stf_off = nullptr;
    int *d_order = nullptr;
    // receivers
    int *d_rec_prob = nullptr;
    long long *d_rec_off = nullptr;
    int *d_rec_comp = nullptr;
    int nrec_total = 0;
    std::vector<int> rec_base;  // per problem: first trace row
    double *d_traces = nullptr;
    int *d_it = nullptr;
    int it = 0;
    void *d_stage = nullptr;
    size_t stage_bytes = 0;
    bool dirty = true;   // device tables need a rebuild
    int ty = TY;         // CTA tile height in rows of 32 columns (autotuned; 4, 8 or 16)
    int l2pf = 0;        // multi-RHS velocity kernel: L2 prefetch distance of its state inputs (autotuned; 0 = off)
    bool own = false;    // every problem gets launches of its own, on BRANCHES parallel streams (autotuned);
                         // false: the single-RHS problems of a family share one persistent launch
    static constexpr int BRANCHES = 4;
    cudaStream_t branch[BRANCHES] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[BRANCHES] = {};
    std::vector<int> branch_of;  // per entry of mr: its branch (balanced by cell-updates)
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 64;
    float last_ms = 0.f;
    int sms = 152;
};

static void free_tables(ewf_batch *b)
{
    for (auto &f : b->fams) {
        cudaFree(f.d_probs);
        cudaFree(f.d_item0);
        f.d_probs = nullptr;
        f.d_item0 = nullptr;
    }
    cudaFree(b->d_all); b->d_all = nullptr;
    cudaFree(b->d_src); b->d_src = nullptr;
    cudaFree(b->d_src_start); b->d_src_start = nullptr;
    cudaFree(b->d_stf); b->d_stf = nullptr;
    cudaFree(b->d_stf_off); b->d_stf_off = nullptr;
    cudaFree(b->d_order); b->d_order = nullptr;
    cudaFree(b->d_rec_prob); b->d_rec_prob = nullptr;
    cudaFree(b->d_rec_off); b->d_rec_off = nullptr;
    cudaFree(b->d_rec_comp); b->d_rec_comp = nullptr;
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
}

extern "C" void ewf_batch_destroy(ewf_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_tables(b);
    for (auto &q : b->probs) {
        for (auto &x : q.state) cudaFree(x);
        for (auto &x : q.mats) cudaFree(x);
        for (auto &x : q.w1) cudaFree(x);
        cudaFree(q.w3);
    }
    cudaFree(b->d_traces);
    cudaFree(b->d_it);
    cudaFree(b->d_stage);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    for (auto &e : b->join_ev)
        if (e) cudaEventDestroy(e);
    for (auto &x : b->branch)
        if (x) cudaStreamDestroy(x);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int ewf_batch_create(int32_t n, const ewf_params *p, const int32_t *n_rhs, ewf_batch **out)
{
    if (!out || !p || n < 1 || n > 4096) return ewf_fail(EWF_ERR_ARG, "bad batch size");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return ewf_fail(EWF_ERR_NODEVICE, "no CUDA device visible");
    }
    for (int i = 0; i < n; ++i) {
        const ewf_params &q = p[i];
        if (q.nx < 4 || q.ny < 4 || q.nz < 4) return ewf_fail(EWF_ERR_ARG, "problem %d: grid must be >= 4", i);
        if (q.precision != EWF_PREC_F32) return ewf_fail(EWF_ERR_UNSUPPORTED, "problem %d: batches are FP32", i);
        if (q.nt != p[0].nt) return ewf_fail(EWF_ERR_ARG, "problem %d: every problem of a batch runs the same nt", i);
        if ((q.model == EWF_MODEL_ISO) != (q.damping == EWF_DAMP_PML1D))
            return ewf_fail(EWF_ERR_UNSUPPORTED, "problem %d: model/damping combination", i);
        if (q.model == EWF_MODEL_ISO_HET || q.vdamp != 0.0)
            return ewf_fail(EWF_ERR_UNSUPPORTED, "problem %d: batches run models 0 and 1 without vdamp", i);
        if (q.nx > q.ny && q.over_y > 0) return ewf_fail(EWF_ERR_UNSUPPORTED, "problem %d: nx > ny with over_y > 0", i);
        if (n_rhs && (n_rhs[i] < 1 || n_rhs[i] > 64)) return ewf_fail(EWF_ERR_ARG, "problem %d: 1..64 right-hand sides", i);
        if (!(q.dx > 0 && q.dy > 0 && q.dz > 0 && q.dt > 0)) return ewf_fail(EWF_ERR_ARG, "problem %d: spacing/dt", i);
    }
    ewf_batch *b = new (std::nothrow) ewf_batch();
    if (!b) return ewf_fail(EWF_ERR_NOMEM, "host allocation");
    cudaGetDevice(&b->device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    b->nt = p[0].nt;
    b->probs.resize(n);
    size_t stage = 0;
#define CKB(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            int s_ = ewf_fail(e_ == cudaErrorMemoryAllocation ? EWF_ERR_NOMEM : EWF_ERR_CUDA,         \
                              "%s: %s", #call, cudaGetErrorString(e_));                              \
            ewf_batch_destroy(b);                                                                    \
            return s_;                                                                               \
        }                                                                                            \
    } while (0)
    CKB(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    CKB(cudaEventCreate(&b->ev0));
    CKB(cudaEventCreate(&b->ev1));
    CKB(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    for (int k = 0; k < ewf_batch::BRANCHES; ++k) {
        CKB(cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking));
        CKB(cudaEventCreateWithFlags(&b->join_ev[k], cudaEventDisableTiming));
    }
    for (int i = 0; i < n; ++i) {
        Prob &q = b->probs[i];
        q.p = p[i];
        q.p.workdir = nullptr;
        q.R = n_rhs ? n_rhs[i] : 1;
        q.kchunk = p[i].kchunk > 0 ? p[i].kchunk : 16;
        if (q.p.model == EWF_MODEL_ORTHO)
            q.fdiv = ewf_fdiv_verified((float)q.p.dx) && ewf_fdiv_verified((float)q.p.dy) &&
                     ewf_fdiv_verified((float)q.p.dz);
        const int hx = 32;
        q.sx = hx + ((q.p.nx + 2 + 31) / 32) * 32;
        q.sy = (long long)q.sx * (q.p.ny + 3);
        q.box = (size_t)q.sy * (q.p.nz + 3);
        q.base_off = hx + (long long)q.sx + q.sy;
        q.sxs = q.sx;
        q.sys = q.sy;
        q.sbox = q.box * q.R;      // R boxes back to back
        q.sbase_off = q.base_off;
        q.src.resize(q.R);
        for (int f = 0; f < 9; ++f) {
            CKB(cudaMalloc(&q.state[f], q.sbox * 4));
            CKB(cudaMemsetAsync(q.state[f], 0, q.sbox * 4, b->stream));
        }
        const int nm = q.p.model == EWF_MODEL_ISO ? 2 : 12;
        for (int f = 0; f < nm; ++f) {
            CKB(cudaMalloc(&q.mats[f], q.box * 4));
            CKB(cudaMemsetAsync(q.mats[f], 0, q.box * 4, b->stream));
        }
        if (q.p.damping == EWF_DAMP_W3D) {
            CKB(cudaMalloc(&q.w3, q.box * 4));
            CKB(cudaMemsetAsync(q.w3, 0, q.box * 4, b->stream));
        } else {
            const int n1[3] = {q.p.nx + 2, q.p.ny + 2, q.p.nz + 2};
            for (int a = 0; a < 3; ++a) {
                CKB(cudaMalloc(&q.w1[a], n1[a] * 4));
                CKB(cudaMemsetAsync(q.w1[a], 0, n1[a] * 4, b->stream));
            }
        }
        stage = std::max(stage, (size_t)(q.p.nx + 1) * (q.p.ny + 1) * (q.p.nz + 1) * 8);
        b->nrhs_total += q.R;
    }
    CKB(cudaMalloc(&b->d_stage, stage));
    b->stage_bytes = stage;
    CKB(cudaMalloc(&b->d_it, sizeof(int)));
    CKB(cudaMemsetAsync(b->d_it, 0, sizeof(int), b->stream));
    CKB(cudaStreamSynchronize(b->stream));
#undef CKB
    *out = b;
    return EWF_OK;
}

static int check_prob(const ewf_batch *b, int32_t prob)
{
    if (!b) return ewf_fail(EWF_ERR_ARG, "NULL batch");
    if (prob < 0 || prob >= (int)b->probs.size()) return ewf_fail(EWF_ERR_ARG, "problem %d out of range", prob);
    return EWF_OK;
}

static int mat_slot(int model, int id)
{
    static const int ortho[] = {EWF_M_C11, EWF_M_C22, EWF_M_C33, EWF_M_C12, EWF_M_C13, EWF_M_C23,
                                EWF_M_C66XY, EWF_M_C55XZ, EWF_M_C44YZ, EWF_M_BX, EWF_M_BY, EWF_M_BZ};
    if (model == EWF_MODEL_ISO) return id == EWF_M_C11 ? 0 : id == EWF_M_C12 ? 1 : -1;
    for (int q = 0; q < 12; ++q)
        if (ortho[q] == id) return q;
    return -1;
}

extern "C" int ewf_batch_set_field(ewf_batch *b, int32_t prob, int32_t field, const void *host, size_t n,
                                   int32_t dtype_bytes)
{
    int st = check_prob(b, prob);
    if (st) return st;
    if (!host || (dtype_bytes != 4 && dtype_bytes != 8)) return ewf_fail(EWF_ERR_ARG, "bad host buffer");
    Prob &q = b->probs[prob];
    int ex, ey, ez;
    if (!ewf_field_extent(q.p, field, &ex, &ey, &ez)) return ewf_fail(EWF_ERR_ARG, "field %d not in this problem", field);
    if (n != (size_t)ex * ey * ez) return ewf_fail(EWF_ERR_ARG, "field %d: %zu elements, %d expected", field, n, ex * ey * ez);
    float *dst;
    int sx = q.sx;
    long long sy = q.sy;
    const int ms = mat_slot(q.p.model, field);
    if (ms >= 0) dst = bptr(q, q.mats[ms]);
    else if (field == EWF_D_W3D) dst = bptr(q, q.w3);
    else if (field >= EWF_D_WX && field <= EWF_D_WZ) { dst = (float *)q.w1[field - EWF_D_WX]; sx = 0; sy = 0; }
    else return ewf_fail(EWF_ERR_ARG, "field %d: batches take materials and damping (state starts at zero)", field);
    CK(cudaMemcpyAsync(b->d_stage, host, n * dtype_bytes, cudaMemcpyHostToDevice, b->stream));
    const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
    if (dtype_bytes == 4) k_pack<float, float><<<nb, 256, 0, b->stream>>>(dst, (const float *)b->d_stage, ex, ey, ez, sx, sy);
    else k_pack<float, double><<<nb, 256, 0, b->stream>>>(dst, (const double *)b->d_stage, ex, ey, ez, sx, sy);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(b->stream));
    if (ms >= 0) q.m_set[ms] = true;
    if (field >= EWF_D_WX && field <= EWF_D_W3D) q.w_set[field - EWF_D_WX] = true;
    return EWF_OK;
}

extern "C" int ewf_batch_set_stf(ewf_batch *b, int32_t prob, const double *stf, size_t n)
{
    int st = check_prob(b, prob);
    if (st) return st;
    if (!stf || n < (size_t)b->nt) return ewf_fail(EWF_ERR_ARG, "Src needs %d samples", b->nt);
    b->probs[prob].stf.assign(stf, stf + b->nt);
    b->dirty = true;
    return EWF_OK;
}

extern "C" int ewf_batch_set_sources(ewf_batch *b, int32_t prob, int32_t rhs, int32_t n, const int32_t *cijk,
                                     const double *coef)
{
    int st = check_prob(b, prob);
    if (st) return st;
    Prob &q = b->probs[prob];
    if (rhs < 0 || rhs >= q.R) return ewf_fail(EWF_ERR_ARG, "rhs %d out of range", rhs);
    if (n < 0 || n > MAXSRC || (n > 0 && (!cijk || !coef))) return ewf_fail(EWF_ERR_ARG, "0..%d sources", MAXSRC);
    std::vector<BatchSrc> v;
    for (int e = 0; e < n; ++e) {
        const int c = cijk[4 * e], i = cijk[4 * e + 1], j = cijk[4 * e + 2], k = cijk[4 * e + 3];
        int ex, ey, ez;
        if (c < EWF_F_SXX || c > EWF_F_SYZ || !ewf_field_extent(q.p, c, &ex, &ey, &ez))
            return ewf_fail(EWF_ERR_ARG, "source %d: not a stress field", e);
        if (i < 0 || j < 0 || k < 0 || i >= ex || j >= ey || k >= ez) return ewf_fail(EWF_ERR_ARG, "source %d outside the grid", e);
        v.push_back(BatchSrc{prob, rhs, c, i, j, k, coef[e]});
    }
    q.src[rhs] = v;
    b->dirty = true;
    return EWF_OK;
}

extern "C" int ewf_batch_set_moment_tensor(ewf_batch *b, int32_t prob, int32_t rhs, const double mt[6], int32_t xs,
                                           int32_t ys, int32_t zs, int32_t stencil)
{
    if (!mt) return ewf_fail(EWF_ERR_ARG, "NULL tensor");
    int32_t cijk[24];
    double coef[6];
    static const int ok4[6][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {3, 3, 1}, {3, 3, 1}, {2, 2, 1}};
    static const int ani[6][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {2, 2, 1}, {-1, 1, 1}, {3, 2, 1}};
    static const int comp[6] = {EWF_F_SXX, EWF_F_SYY, EWF_F_SZZ, EWF_F_SXY, EWF_F_SXZ, EWF_F_SYZ};
    // statement order of the reference: OK4:336-342 (xx yy zz yz xz xy), ANISO:233-247 (xx yy zz xy yz xz)
    static const int ord_ok4[6] = {0, 1, 2, 5, 4, 3};
    static const int ord_ani[6] = {0, 1, 2, 3, 5, 4};
    if (stencil != 0 && stencil != 1) return ewf_fail(EWF_ERR_ARG, "stencil must be 0 or 1");
    for (int e = 0; e < 6; ++e) {
        const int m = stencil == 0 ? ord_ok4[e] : ord_ani[e];
        const int *o = stencil == 0 ? ok4[m] : ani[m];
        cijk[4 * e] = comp[m];
        cijk[4 * e + 1] = xs + o[0];
        cijk[4 * e + 2] = ys + o[1];
        cijk[4 * e + 3] = zs + o[2];
        coef[e] = mt[m];
    }
    return ewf_batch_set_sources(b, prob, rhs, 6, cijk, coef);
}

extern "C" int ewf_batch_set_receivers(ewf_batch *b, int32_t prob, int32_t n, const int32_t *ijkc)
{
    int st = check_prob(b, prob);
    if (st) return st;
    Prob &q = b->probs[prob];
    if (n < 0 || (n > 0 && !ijkc)) return ewf_fail(EWF_ERR_ARG, "bad receiver list");
    for (int r = 0; r < n; ++r) {
        const int i = ijkc[4 * r], j = ijkc[4 * r + 1], k = ijkc[4 * r + 2], c = ijkc[4 * r + 3];
        int ex, ey, ez;
        if (c < 0 || c > 8 || !ewf_field_extent(q.p, c, &ex, &ey, &ez)) return ewf_fail(EWF_ERR_ARG, "receiver %d field", r);
        if (i < 0 || j < 0 || k < 0 || i >= ex || j >= ey || k >= ez) return ewf_fail(EWF_ERR_ARG, "receiver %d outside", r);
    }
    q.rec.assign(ijkc, ijkc + 4 * (size_t)n);
    b->dirty = true;
    return EWF_OK;
}

template <typename K>
static int persistent_grid(K kernel, int sms, int nitems, int ty)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TX * ty, 0);
    return std::max(1, std::min(nitems, sms * std::max(1, per_sm)));
}

template <int MODEL, int DAMP>
static int family_grid_t(bool stress, int sms, int items, int ty)
{
    return stress ? persistent_grid(k_bstress<float, MODEL, DAMP>, sms, items, ty)
                  : persistent_grid(k_bvelocity<float, MODEL, DAMP>, sms, items, ty);
}

template <bool STRESS>
static int family_grid(const Family &f, int sms, int items)
{
    if (f.model == EWF_MODEL_ISO) return family_grid_t<MODEL_ISO, DAMP_PML1D>(STRESS, sms, items, f.ty);
    if (f.damping == EWF_DAMP_W3D) return family_grid_t<MODEL_ORTHO, DAMP_W3D>(STRESS, sms, items, f.ty);
    return family_grid_t<MODEL_ORTHO, DAMP_SEP>(STRESS, sms, items, f.ty);
}

template <int MODEL, int DAMP>
static void launch_family_t(const Family &f, bool stress, cudaStream_t s)
{
    if (stress)
        k_bstress<float, MODEL, DAMP><<<f.grid_stress, dim3(TX, f.ty), 0, s>>>(f.d_probs, f.d_item0, (int)f.probs.size(),
                                                                               f.nitems);
    else
        k_bvelocity<float, MODEL, DAMP><<<f.grid_vel, dim3(TX, f.ty), 0, s>>>(f.d_probs, f.d_item0, (int)f.probs.size(),
                                                                              f.nitems);
}

static void launch_family(const Family &f, bool stress, cudaStream_t s)
{
    if (f.model == EWF_MODEL_ISO) launch_family_t<MODEL_ISO, DAMP_PML1D>(f, stress, s);
    else if (f.damping == EWF_DAMP_W3D) launch_family_t<MODEL_ORTHO, DAMP_W3D>(f, stress, s);
    else launch_family_t<MODEL_ORTHO, DAMP_SEP>(f, stress, s);
}

// Rebuilds the device tables (problem descriptors, work lists, sources, receivers, traces).
static int build_tables(ewf_batch *b)
{
    CK(cudaStreamSynchronize(b->stream));
    free_tables(b);
    const int n = (int)b->probs.size();
    std::vector<BatchProb<float>> all(n);
    for (int i = 0; i < n; ++i) {
        Prob &q = b->probs[i];
        const ewf_params &p = q.p;
        BatchProb<float> &bp = all[i];
        memset(&bp, 0, sizeof(bp));
        StepArgs<float> &d = bp.a;
        for (int f = 0; f < 9; ++f) d.f[f] = sptr(q, q.state[f]);
        for (int f = 0; f < 12; ++f) d.m[f] = bptr(q, q.mats[f]);
        for (int a = 0; a < 3; ++a) d.w1[a] = (const float *)q.w1[a];
        d.w3 = bptr(q, q.w3);
        d.sy = q.sy;
        d.sx = q.sx;
        d.R = 1;
        d.sxs = q.sx;
        d.sys = q.sy;
        bp.rhs_stride = (long long)q.box;
        bp.R = q.R;
        d.nx = p.nx; d.ny = p.ny; d.nz = p.nz;
        d.bc1_rows = std::min(p.ny, std::min(p.nx, p.ny + std::max(0, p.over_y)));
        d.kchunk = q.kchunk;
        d.dt = (float)p.dt;
        d.rdt = 1.0f / d.dt;
        d.dx = (float)p.dx; d.dy = (float)p.dy; d.dz = (float)p.dz;
        d.rdx = 1.0f / d.dx; d.rdy = 1.0f / d.dy; d.rdz = 1.0f / d.dz;
        d.c66 = (float)p.c66; d.bx = (float)p.bx; d.by = (float)p.by; d.bz = (float)p.bz;
        d.third = 1.0f / 3.0f;
        d.fdiv = q.fdiv ? 1 : 0;
        d.bc1 = p.free_surface == EWF_FS_BC1 ? 1 : 0;
        d.smu_on = p.surface_mu > 0.0 ? 1 : 0;
        d.smu = (float)p.surface_mu;
        d.l2pf = (q.R > 1 || b->own) ? b->l2pf : 0;
        bp.tiles_x = (p.nx + TX - 1) / TX;
        bp.tiles_y = (p.ny + b->ty - 1) / b->ty;
        bp.chunks = (p.nz + q.kchunk - 1) / q.kchunk;
    }
    // families (single-RHS problems sharing one persistent launch) and their work lists;
    // problems with several RHS get their own launches (k_stress_mr / k_velocity_mr)
    b->fams.clear();
    b->mr.clear();
    std::map<std::pair<int, int>, int> fam_of;
    for (int i = 0; i < n; ++i) {
        if (b->probs[i].R > 1 || b->own) {
            b->mr.push_back(i);
            continue;
        }
        const auto key = std::make_pair(b->probs[i].p.model, b->probs[i].p.damping);
        if (!fam_of.count(key)) {
            fam_of[key] = (int)b->fams.size();
            b->fams.push_back(Family{key.first, key.second});
            b->fams.back().ty = b->ty;
        }
        b->fams[fam_of[key]].probs.push_back(i);
    }
    // branches of the own launches: largest problems first, each to the least loaded branch
    b->branch_of.assign(b->mr.size(), 0);
    {
        std::vector<int> idx(b->mr.size());
        for (size_t e = 0; e < idx.size(); ++e) idx[e] = (int)e;
        auto work = [&](int e) {
            const Prob &q = b->probs[b->mr[e]];
            return (double)q.p.nx * q.p.ny * q.p.nz * q.R;
        };
        std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return work(x) > work(y); });
        double load[ewf_batch::BRANCHES] = {};
        for (int e : idx) {
            const int k = (int)(std::min_element(load, load + ewf_batch::BRANCHES) - load);
            b->branch_of[e] = k;
            load[k] += work(e);
        }
    }
    for (auto &f : b->fams) {
        std::vector<BatchProb<float>> v;
        std::vector<int> item0;
        int items = 0;
        for (int i : f.probs) {
            BatchProb<float> d = all[i];
            d.item0 = items;
            item0.push_back(items);
            items += d.tiles_x * d.tiles_y * d.chunks * d.R;
            v.push_back(d);
        }
        f.nitems = items;
        CK(cudaMalloc(&f.d_probs, v.size() * sizeof(BatchProb<float>)));
        CK(cudaMemcpy(f.d_probs, v.data(), v.size() * sizeof(BatchProb<float>), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&f.d_item0, item0.size() * sizeof(int)));
        CK(cudaMemcpy(f.d_item0, item0.data(), item0.size() * sizeof(int), cudaMemcpyHostToDevice));
        f.grid_stress = family_grid<true>(f, b->sms, items);
        f.grid_vel = family_grid<false>(f, b->sms, items);
    }
    CK(cudaMalloc(&b->d_all, n * sizeof(BatchProb<float>)));
    for (int i = 0; i < n; ++i) all[i].item0 = 0;
    b->h_all = all;
    CK(cudaMemcpy(b->d_all, all.data(), n * sizeof(BatchProb<float>), cudaMemcpyHostToDevice));
    // sources grouped by (problem, rhs)
    std::vector<BatchSrc> src;
    std::vector<int> start;
    std::vector<double> stf((size_t)n * b->nt, 0.0);
    std::vector<int> stf_off(n), order(n);
    for (int i = 0; i < n; ++i) {
        Prob &q = b->probs[i];
        for (int r = 0; r < q.R; ++r) {
            start.push_back((int)src.size());
            for (auto &e : q.src[r]) src.push_back(e);
            if (!q.src[r].empty() && q.stf.empty()) return ewf_fail(EWF_ERR_STATE, "problem %d has sources but no Src", i);
        }
        stf_off[i] = i * b->nt;
        if (!q.stf.empty()) std::copy(q.stf.begin(), q.stf.end(), stf.begin() + (size_t)i * b->nt);
        order[i] = q.p.src_order;
    }
    start.push_back((int)src.size());
    b->ngroups = (int)start.size() - 1;
    if (!src.empty()) {
        CK(cudaMalloc(&b->d_src, src.size() * sizeof(BatchSrc)));
        CK(cudaMemcpy(b->d_src, src.data(), src.size() * sizeof(BatchSrc), cudaMemcpyHostToDevice));
    }
    CK(cudaMalloc(&b->d_src_start, start.size() * sizeof(int)));
    CK(cudaMemcpy(b->d_src_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&b->d_stf, stf.size() * sizeof(double)));
    CK(cudaMemcpy(b->d_stf, stf.data(), stf.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&b->d_stf_off, n * sizeof(int)));
    CK(cudaMemcpy(b->d_stf_off, stf_off.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&b->d_order, n * sizeof(int)));
    CK(cudaMemcpy(b->d_order, order.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    // receivers: per problem, RHS-major
    std::vector<int> rp, rc;
    std::vector<long long> ro;
    b->rec_base.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        Prob &q = b->probs[i];
        b->rec_base[i] = (int)rp.size();
        const int nr = (int)q.rec.size() / 4;
        for (int r = 0; r < q.R; ++r)
            for (int e = 0; e < nr; ++e) {
                rp.push_back(i);
                rc.push_back(q.rec[4 * e + 3]);
                ro.push_back((long long)q.rec[4 * e] + (long long)q.rec[4 * e + 1] * q.sx +
                             (long long)q.rec[4 * e + 2] * q.sy + (long long)r * (long long)q.box);
            }
    }
    const int nrec = (int)rp.size();
    if (nrec != b->nrec_total || !b->d_traces) {
        cudaFree(b->d_traces);
        b->d_traces = nullptr;
        if (nrec) {
            CK(cudaMalloc(&b->d_traces, (size_t)nrec * b->nt * sizeof(double)));
            CK(cudaMemset(b->d_traces, 0, (size_t)nrec * b->nt * sizeof(double)));
        }
    }
    b->nrec_total = nrec;
    if (nrec) {
        CK(cudaMalloc(&b->d_rec_prob, nrec * sizeof(int)));
        CK(cudaMemcpy(b->d_rec_prob, rp.data(), nrec * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&b->d_rec_comp, nrec * sizeof(int)));
        CK(cudaMemcpy(b->d_rec_comp, rc.data(), nrec * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMalloc(&b->d_rec_off, nrec * sizeof(long long)));
        CK(cudaMemcpy(b->d_rec_off, ro.data(), nrec * sizeof(long long), cudaMemcpyHostToDevice));
    }
    b->dirty = false;
    return EWF_OK;
}

template <int MODEL, int DAMP>
static void launch_mr_t(const BatchProb<float> &p, int ty, bool stress, cudaStream_t s)
{
    const dim3 grd(p.tiles_x * p.R, p.tiles_y, p.chunks);
    if (stress)
        k_stress_mr<float, MODEL, DAMP><<<grd, dim3(TX, ty), 0, s>>>(p.a, p.R, p.rhs_stride);
    else
        k_velocity_mr<float, MODEL, DAMP><<<grd, dim3(TX, ty), 0, s>>>(p.a, p.R, p.rhs_stride);
}

static void launch_mr(const ewf_batch *b, int i, bool stress, cudaStream_t s)
{
    const ewf_params &q = b->probs[i].p;
    const BatchProb<float> &p = b->h_all[i];
    if (q.model == EWF_MODEL_ISO) launch_mr_t<MODEL_ISO, DAMP_PML1D>(p, b->ty, stress, s);
    else if (q.damping == EWF_DAMP_W3D) launch_mr_t<MODEL_ORTHO, DAMP_W3D>(p, b->ty, stress, s);
    else launch_mr_t<MODEL_ORTHO, DAMP_SEP>(p, b->ty, stress, s);
}

static void batch_step(ewf_batch *b, cudaEvent_t *ev)
{
    cudaStream_t s = b->stream;
    if (ev) cudaEventRecord(ev[0], s);
    // the own launches of one phase: on one stream, or forked over the branch streams and joined
    auto own_phase = [&](bool stress) {
        if (!b->own || b->mr.size() < 2) {
            for (int i : b->mr) launch_mr(b, i, stress, s);
            return;
        }
        cudaEventRecord(b->fork_ev, s);
        for (auto &x : b->branch) cudaStreamWaitEvent(x, b->fork_ev, 0);
        for (size_t e = 0; e < b->mr.size(); ++e) launch_mr(b, b->mr[e], stress, b->branch[b->branch_of[e]]);
        for (int k = 0; k < ewf_batch::BRANCHES; ++k) {
            cudaEventRecord(b->join_ev[k], b->branch[k]);
            cudaStreamWaitEvent(s, b->join_ev[k], 0);
        }
    };
    own_phase(true);
    for (auto &f : b->fams) launch_family(f, true, s);
    if (ev) cudaEventRecord(ev[1], s);
    if (b->d_src)
        k_binject<float><<<(b->ngroups + 127) / 128, 128, 0, s>>>(b->d_all, b->d_src, b->d_src_start, b->ngroups, b->d_stf,
                                                                  b->d_stf_off, b->d_order, b->nt, b->d_it);
    if (ev) cudaEventRecord(ev[2], s);
    own_phase(false);
    for (auto &f : b->fams) launch_family(f, false, s);
    if (ev) cudaEventRecord(ev[3], s);
    if (b->nrec_total)
        k_brecord<float><<<std::min((b->nrec_total + 255) / 256, 1024), 256, 0, s>>>(b->d_all, b->d_rec_prob, b->d_rec_off,
                                                                                   b->d_rec_comp, b->nrec_total, b->d_traces, b->nt, b->d_it);
    k_advance<<<1, 1, 0, s>>>(b->d_it);
    if (ev) cudaEventRecord(ev[4], s);
}

static int batch_ready(ewf_batch *b)
{
    for (size_t i = 0; i < b->probs.size(); ++i) {
        const Prob &q = b->probs[i];
        const int nm = q.p.model == EWF_MODEL_ISO ? 2 : 12;
        for (int f = 0; f < nm; ++f)
            if (!q.m_set[f]) return ewf_fail(EWF_ERR_STATE, "problem %zu: material slot %d not set", i, f);
        if (q.p.damping == EWF_DAMP_W3D ? !q.w_set[3] : !(q.w_set[0] && q.w_set[1] && q.w_set[2]))
            return ewf_fail(EWF_ERR_STATE, "problem %zu: damping not set", i);
    }
    if (b->dirty) return build_tables(b);
    return EWF_OK;
}

extern "C" int ewf_batch_reset(ewf_batch *b)
{
    if (!b) return ewf_fail(EWF_ERR_ARG, "NULL batch");
    for (auto &q : b->probs)
        for (auto &x : q.state) CK(cudaMemsetAsync(x, 0, q.sbox * 4, b->stream));
    if (b->d_traces) CK(cudaMemsetAsync(b->d_traces, 0, (size_t)b->nrec_total * b->nt * sizeof(double), b->stream));
    CK(cudaMemsetAsync(b->d_it, 0, sizeof(int), b->stream));
    CK(cudaStreamSynchronize(b->stream));
    b->it = 0;
    return EWF_OK;
}

extern "C" int ewf_batch_run(ewf_batch *b, int32_t nsteps)
{
    if (!b || nsteps < 0) return ewf_fail(EWF_ERR_ARG, "bad argument");
    int st = batch_ready(b);
    if (st) return st;
    if (b->it + nsteps > b->nt) return ewf_fail(EWF_ERR_ARG, "step %d + %d exceeds nt = %d", b->it, nsteps, b->nt);
    const bool use_graph = b->gsteps > 0 && nsteps >= b->gsteps;
    if (use_graph && !b->gexec) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        for (int s = 0; s < b->gsteps; ++s) batch_step(b, nullptr);
        const cudaError_t le = cudaGetLastError();
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return ewf_fail(EWF_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(le != cudaSuccess ? le : ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->gexec = nullptr;
            return ewf_fail(EWF_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ie));
        }
    }
    CK(cudaEventRecord(b->ev0, b->stream));
    int done = 0;
    if (use_graph)
        for (; done + b->gsteps <= nsteps; done += b->gsteps) CK(cudaGraphLaunch(b->gexec, b->stream));
    for (; done < nsteps; ++done) batch_step(b, nullptr);
    CK(cudaGetLastError());
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1));
    b->it += nsteps;
    return EWF_OK;
}

extern "C" int ewf_batch_last_run_ms(const ewf_batch *b, double *ms)
{
    if (!b || !ms) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *ms = b->last_ms;
    return EWF_OK;
}

extern "C" int ewf_batch_get_seismograms(ewf_batch *b, int32_t prob, int32_t rhs, double *out, size_t n)
{
    int st = check_prob(b, prob);
    if (st) return st;
    const Prob &q = b->probs[prob];
    if (rhs < 0 || rhs >= q.R) return ewf_fail(EWF_ERR_ARG, "rhs out of range");
    const int nr = (int)q.rec.size() / 4;
    if (n != (size_t)nr * b->nt || (!out && n)) return ewf_fail(EWF_ERR_ARG, "%zu samples, %d expected", n, nr * b->nt);
    if (b->dirty) return ewf_fail(EWF_ERR_STATE, "receivers changed since the last run");
    if (n)
        CK(cudaMemcpy(out, b->d_traces + ((size_t)b->rec_base[prob] + (size_t)rhs * nr) * b->nt, n * sizeof(double),
                      cudaMemcpyDeviceToHost));
    return EWF_OK;
}

extern "C" int ewf_batch_get_field(ewf_batch *b, int32_t prob, int32_t rhs, int32_t field, void *host, size_t n,
                                   int32_t dtype_bytes)
{
    int st = check_prob(b, prob);
    if (st) return st;
    const Prob &q = b->probs[prob];
    if (rhs < 0 || rhs >= q.R || field < 0 || field > 8 || !host || (dtype_bytes != 4 && dtype_bytes != 8))
        return ewf_fail(EWF_ERR_ARG, "bad argument");
    int ex, ey, ez;
    ewf_field_extent(q.p, field, &ex, &ey, &ez);
    if (n != (size_t)ex * ey * ez) return ewf_fail(EWF_ERR_ARG, "field size");
    const float *src = sptr(q, q.state[field]) + (size_t)rhs * q.box;
    const unsigned nb = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16);
    if (dtype_bytes == 4) k_unpack<float, float><<<nb, 256, 0, b->stream>>>((float *)b->d_stage, src, ex, ey, ez, q.sx, q.sy);
    else k_unpack<double, float><<<nb, 256, 0, b->stream>>>((double *)b->d_stage, src, ex, ey, ez, q.sx, q.sy);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, b->d_stage, n * dtype_bytes, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return EWF_OK;
}

// Times `nsteps` steps for each (tile height, z-chunk) candidate with CUDA events, keeps the
// fastest, and leaves the batch reset (the tuning steps advance the state).
extern "C" int ewf_batch_autotune(ewf_batch *b, int32_t nsteps, int32_t *kchunk_out)
{
    if (!b || nsteps < 1) return ewf_fail(EWF_ERR_ARG, "bad argument");
    static const int cand[] = {8, 12, 16, 24, 32, 48, 64};
    static const int ty_cand[] = {4, 8, 16};
    float best = 1e30f;
    int best_k = 16, best_ty = b->ty;
    bool best_own = b->own;
    cudaEvent_t ev[5];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int own = 0; own < 2; ++own)
    for (int ty : ty_cand)
    for (int kc : cand) {
        for (auto &q : b->probs) q.kchunk = std::max(4, std::min(kc, q.p.nz));
        b->ty = ty;
        b->own = own != 0;
        b->dirty = true;
        int st = batch_ready(b);
        if (st) { for (auto &e : ev) cudaEventDestroy(e); return st; }
        st = ewf_batch_reset(b);
        if (st) { for (auto &e : ev) cudaEventDestroy(e); return st; }
        batch_step(b, nullptr);  // warm
        CK(cudaEventRecord(b->ev0, b->stream));
        for (int s = 1; s < std::min(nsteps + 1, b->nt); ++s) batch_step(b, nullptr);
        CK(cudaEventRecord(b->ev1, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
        if (ms < best) { best = ms; best_k = kc; best_ty = ty; best_own = own != 0; }
    }
    for (auto &q : b->probs) q.kchunk = std::max(4, std::min(best_k, q.p.nz));
    b->ty = best_ty;
    b->own = best_own;
    b->dirty = true;
    if (int st = batch_ready(b)) { for (auto &e : ev) cudaEventDestroy(e); return st; }
    // then the multi-RHS velocity kernel's L2 prefetch distance at that setting
    int best_pf = 0;
    if (!b->mr.empty()) {
        static const int pf_cand[] = {0, 2, 3, 4};
        float best_pf_ms = 1e30f;
        for (int pf : pf_cand) {
            b->l2pf = pf;
            b->dirty = true;
            int st = batch_ready(b);
            if (!st) st = ewf_batch_reset(b);
            if (st) { for (auto &e : ev) cudaEventDestroy(e); return st; }
            batch_step(b, nullptr);  // warm
            CK(cudaEventRecord(b->ev0, b->stream));
            for (int s = 1; s < std::min(nsteps + 1, b->nt); ++s) batch_step(b, nullptr);
            CK(cudaEventRecord(b->ev1, b->stream));
            CK(cudaStreamSynchronize(b->stream));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            if (ms < best_pf_ms) { best_pf_ms = ms; best_pf = pf; }
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    b->l2pf = best_pf;
    b->dirty = true;
    int st = batch_ready(b);
    if (st) return st;
    if (kchunk_out) *kchunk_out = best_k;
    return ewf_batch_reset(b);
}

extern "C" int ewf_batch_set_tile(ewf_batch *b, int32_t tile_y)
{
    if (!b) return ewf_fail(EWF_ERR_ARG, "NULL batch");
    if (tile_y != 4 && tile_y != 8 && tile_y != 16) return ewf_fail(EWF_ERR_ARG, "tile_y must be 4, 8 or 16 (got %d)", tile_y);
    b->ty = tile_y;
    b->dirty = true;
    return EWF_OK;
}

extern "C" int ewf_batch_set_launch(ewf_batch *b, int32_t own)
{
    if (!b) return ewf_fail(EWF_ERR_ARG, "NULL batch");
    if (own != 0 && own != 1) return ewf_fail(EWF_ERR_ARG, "own must be 0 or 1 (got %d)", own);
    b->own = own != 0;
    b->dirty = true;
    return EWF_OK;
}

extern "C" int ewf_batch_get_launch(const ewf_batch *b, int32_t *own)
{
    if (!b || !own) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *own = b->own ? 1 : 0;
    return EWF_OK;
}

extern "C" int ewf_batch_set_l2_prefetch(ewf_batch *b, int32_t planes)
{
    if (!b) return ewf_fail(EWF_ERR_ARG, "NULL batch");
    if (planes < 0 || planes > 8) return ewf_fail(EWF_ERR_ARG, "planes must be in [0, 8] (got %d)", planes);
    b->l2pf = planes;
    b->dirty = true;
    return EWF_OK;
}

extern "C" int ewf_batch_get_l2_prefetch(const ewf_batch *b, int32_t *planes)
{
    if (!b || !planes) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *planes = b->l2pf;
    return EWF_OK;
}

extern "C" int ewf_batch_get_tile(const ewf_batch *b, int32_t *tile_y)
{
    if (!b || !tile_y) return ewf_fail(EWF_ERR_ARG, "NULL argument");
    *tile_y = b->ty;
    return EWF_OK;
}
