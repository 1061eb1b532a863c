// C-ABI entry points (include/dcf.h).  Every call validates its arguments on the
// host, enqueues kernels on the context's stream and only synchronises when it
// must hand data back to host memory; device-side failures (loop bounds) are
// collected in a device error word and reported by the next synchronising call.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <string>

#include "../../include/dcf.h"
#include "dcf_kernels.cuh"

using namespace dcf;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct ProfEvent {
    cudaEvent_t ev;
    int id;
    bool begin;
};

struct dcf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int sm_count = 0;
    unsigned *d_err = nullptr;        // device error bits
    unsigned *d_stats = nullptr;      // kmin, kmax, nans (per build; tree copies what it needs)
    char last_error[512] = {0};
    uint64_t launches = 0;
    int up_steps = 2048;              // bottom-up fold steps per walker before pointer jumping
    int tile2d[2] = {64, 64};         // build tile of 2-D images (width, height)
    int tile3d[3] = {16, 16, 16};     // build tile of 3-D images
    int level_sync = 1;               // barrier between band-merge levels inside a tile
    std::mutex trees_mu;
    std::set<dcf_tree *> trees;       // live trees; orphaned (stream cleared) when the context goes
    DevBuf scratch[12];               // reusable work buffers (filter, spectra, attributes)
    bool prof_on = false;
    ProfEvent *prof_ev = nullptr;     // recorded events, in launch order
    int prof_n = 0, prof_cap = 0;
    double prof_ms[P_COUNT] = {0};
    uint64_t prof_cnt[P_COUNT] = {0};
};

// the context whose API call is running on this thread (for prof_begin/prof_end)
static thread_local dcf_ctx *t_active = nullptr;
struct ActiveScope {
    dcf_ctx *prev;
    explicit ActiveScope(dcf_ctx *c) : prev(t_active) { t_active = c; }
    ~ActiveScope() { t_active = prev; }
};

static void prof_record(int id, bool begin, cudaStream_t s)
{
    dcf_ctx *c = t_active;
    if (!c || !c->prof_on) return;
    if (c->prof_n == c->prof_cap) {
        int cap = c->prof_cap ? 2 * c->prof_cap : 256;
        ProfEvent *nv = (ProfEvent *)realloc(c->prof_ev, cap * sizeof(ProfEvent));
        if (!nv) return;
        for (int i = c->prof_cap; i < cap; i++) cudaEventCreate(&nv[i].ev);
        c->prof_ev = nv;
        c->prof_cap = cap;
    }
    ProfEvent &e = c->prof_ev[c->prof_n++];
    e.id = id;
    e.begin = begin;
    cudaEventRecord(e.ev, s);
}

namespace dcf {
void prof_begin(int id, cudaStream_t s) { prof_record(id, true, s); }
void prof_end(int id, cudaStream_t s) { prof_record(id, false, s); }
}  // namespace dcf

// fold recorded event pairs into per-kernel totals
static void prof_collect(dcf_ctx *c)
{
    if (!c->prof_n) return;
    cudaStreamSynchronize(c->stream);
    int open[P_COUNT];
    for (int i = 0; i < P_COUNT; i++) open[i] = -1;
    for (int i = 0; i < c->prof_n; i++) {
        ProfEvent &e = c->prof_ev[i];
        if (e.begin) {
            open[e.id] = i;
        } else if (open[e.id] >= 0) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, c->prof_ev[open[e.id]].ev, e.ev);
            c->prof_ms[e.id] += ms;
            c->prof_cnt[e.id]++;
            open[e.id] = -1;
        }
    }
    c->prof_n = 0;
}

struct dcf_tree {
    dcf_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;           // buffers are freed in this stream's order
    Geom g{};
    int dtype = 0;
    bool tree_min = false;
    float pixdim[3] = {1, 1, 1};
    float *gval = nullptr;
    int *parent = nullptr;
    unsigned char *isroot = nullptr;
    unsigned *stats = nullptr;               // kmin, kmax, nans of the input
    unsigned long long *num_nodes = nullptr;
    AttrBufs attr;
    int attr_idx = -1;
    void *attr_mem = nullptr;                // one allocation for all record arrays
};

// attribute -> group (attributes.c:1224-1248; 18 = bbox elongation, extent group)
static const int ATTR_GROUP[DCF_NUM_ATTRIBUTES] = {0, 1, 1, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4, 1};

static dcf_status set_err(dcf_ctx *c, dcf_status s, const char *fmt, ...)
{
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->last_error, sizeof(c->last_error), fmt, ap);
        va_end(ap);
    }
    return s;
}

#define CU(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess) return set_err(ctx, _e == cudaErrorMemoryAllocation ? DCF_ERR_NOMEM : DCF_ERR_CUDA, \
                                              "%s: %s", #call, cudaGetErrorString(_e));                  \
    } while (0)

static dcf_status check_launch(dcf_ctx *ctx, int nlaunch)
{
    ctx->launches += (uint64_t)nlaunch;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(ctx, DCF_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    return DCF_OK;
}

// synchronise the stream, then turn device error bits into a status
static dcf_status sync_and_check(dcf_ctx *ctx)
{
    CU(cudaStreamSynchronize(ctx->stream));
    unsigned err = 0;
    CU(cudaMemcpy(&err, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (err) {
        CU(cudaMemset(ctx->d_err, 0, sizeof(unsigned)));
        return set_err(ctx, DCF_ERR_TIMEOUT, "device loop bound exceeded (bits 0x%x)", err);
    }
    return DCF_OK;
}

static dcf_status scratch(dcf_ctx *ctx, int slot, size_t bytes, void **out)
{
    DevBuf &b = ctx->scratch[slot];
    if (b.bytes < bytes) {
        if (b.p) CU(cudaFree(b.p));
        b.p = nullptr;
        b.bytes = 0;
        CU(cudaMalloc(&b.p, bytes));
        b.bytes = bytes;
    }
    *out = b.p;
    return DCF_OK;
}

// stream-ordered free, or a synchronous one for a tree whose context is gone
static void dev_free(void *p, cudaStream_t s)
{
    if (!p) return;
    if (s) cudaFreeAsync(p, s);
    else cudaFree(p);
}

static void orphan_tree(dcf_tree *t)
{
    t->ctx = nullptr;
    t->stream = nullptr;
}

extern "C" {

const char *dcf_status_string(dcf_status s)
{
    switch (s) {
    case DCF_OK: return "ok";
    case DCF_ERR_INVALID: return "invalid argument";
    case DCF_ERR_NOMEM: return "out of memory";
    case DCF_ERR_CUDA: return "CUDA error";
    case DCF_ERR_TIMEOUT: return "device loop bound exceeded";
    case DCF_ERR_NAN: return "image contains NaN";
    case DCF_ERR_STATE: return "invalid state";
    case DCF_ERR_IO: return "I/O error";
    case DCF_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

dcf_status dcf_ctx_create(int device, void *cuda_stream, dcf_ctx **out)
{
    if (!out) return DCF_ERR_INVALID;
    *out = nullptr;
    dcf_ctx *ctx = new (std::nothrow) dcf_ctx();
    if (!ctx) return DCF_ERR_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        delete ctx;
        return DCF_ERR_CUDA;
    }
    if (cuda_stream) {
        ctx->stream = (cudaStream_t)cuda_stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return DCF_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (const char *e = getenv("DCF_TILE2D")) {  // e.g. "32x32"
        int a = 0, b = 0;
        if (sscanf(e, "%dx%d", &a, &b) == 2 && a > 0 && b > 0 && a * b <= TILE_MAX_PIX) {
            ctx->tile2d[0] = a;
            ctx->tile2d[1] = b;
        }
    }
    if (const char *e = getenv("DCF_LEVEL_SYNC")) ctx->level_sync = atoi(e) != 0;
    if (const char *e = getenv("DCF_UP_STEPS")) {
        int v = atoi(e);
        if (v >= 0 && v < (1 << 20)) ctx->up_steps = v;
    }
    // keep freed tree buffers in the device's default pool: repeated builds then
    // allocate stream-ordered without cudaMalloc's cost or its implicit sync
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (cudaMalloc(&ctx->d_err, 4 * sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(ctx->d_err, 0, 4 * sizeof(unsigned)) != cudaSuccess) {
        if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return DCF_ERR_NOMEM;
    }
    *out = ctx;
    return DCF_OK;
}

dcf_status dcf_ctx_destroy(dcf_ctx *ctx)
{
    if (!ctx) return DCF_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
    {
        // trees that outlive their context free their buffers synchronously later
        std::lock_guard<std::mutex> lk(ctx->trees_mu);
        for (dcf_tree *t : ctx->trees) orphan_tree(t);
        ctx->trees.clear();
    }
    for (auto &b : ctx->scratch)
        if (b.p) cudaFree(b.p);
    for (int i = 0; i < ctx->prof_cap; i++) cudaEventDestroy(ctx->prof_ev[i].ev);
    free(ctx->prof_ev);
    cudaFree(ctx->d_err);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return DCF_OK;
}

dcf_status dcf_ctx_synchronize(dcf_ctx *ctx)
{
    if (!ctx) return DCF_ERR_INVALID;
    return sync_and_check(ctx);
}

const char *dcf_ctx_last_error(const dcf_ctx *ctx) { return ctx ? ctx->last_error : "no context"; }

uint64_t dcf_ctx_launch_count(const dcf_ctx *ctx) { return ctx ? ctx->launches : 0; }

dcf_status dcf_ctx_set_profiling(dcf_ctx *ctx, int enable)
{
    if (!ctx) return DCF_ERR_INVALID;
    prof_collect(ctx);
    ctx->prof_on = enable != 0;
    for (int i = 0; i < P_COUNT; i++) {
        ctx->prof_ms[i] = 0.0;
        ctx->prof_cnt[i] = 0;
    }
    return DCF_OK;
}

int dcf_profile_num_kernels(void) { return P_COUNT; }

const char *dcf_profile_kernel_name(int id)
{
    static const char *names[P_COUNT] = {"stats", "tile_build", "seam_merge", "canonicalise", "attr_pixels",
                                         "attr_bottom_up", "attr_pointer_jump", "filter_flag", "filter_resolve", "filter_jump",
                                         "filter_out", "check", "spectrum", "copy", "batch", "adjoint"};
    return (id >= 0 && id < P_COUNT) ? names[id] : "?";
}

dcf_status dcf_ctx_profile(dcf_ctx *ctx, int id, double *total_ms, uint64_t *launches)
{
    if (!ctx || id < 0 || id >= P_COUNT) return DCF_ERR_INVALID;
    prof_collect(ctx);
    if (total_ms) *total_ms = ctx->prof_ms[id];
    if (launches) *launches = ctx->prof_cnt[id];
    return DCF_OK;
}

static void free_attr(dcf_tree *t)
{
    dev_free(t->attr_mem, t->stream);
    t->attr_mem = nullptr;
    t->attr = AttrBufs();
    t->attr_idx = -1;
}

dcf_status dcf_tree_destroy(dcf_tree *t)
{
    if (!t) return DCF_ERR_INVALID;
    // stream-ordered frees: the memory returns to the pool once queued work is done.
    // Trees must be destroyed before their context.
    if (t->ctx) {
        std::lock_guard<std::mutex> lk(t->ctx->trees_mu);
        t->ctx->trees.erase(t);
    }
    free_attr(t);
    dev_free(t->gval, t->stream);
    dev_free(t->parent, t->stream);
    dev_free(t->isroot, t->stream);
    dev_free(t->stats, t->stream);
    delete t;
    return DCF_OK;
}

static TreeView view_of(const dcf_tree *t)
{
    TreeView v;
    v.g = t->g;
    v.tree_min = t->tree_min;
    v.kmax = t->stats + 1;
    v.gval = t->gval;
    v.parent = t->parent;
    v.isroot = t->isroot;
    for (int i = 0; i < 3; i++) v.pixdim[i] = t->pixdim[i];
    v.integer_levels = t->dtype == U8 || t->dtype == U16;
    return v;
}

// allocate and accumulate the records of attr_idx's group
static dcf_status compute_attributes(dcf_ctx *ctx, dcf_tree *t, int attr_idx)
{
    const int group = ATTR_GROUP[attr_idx];
    if (t->attr_mem && t->attr.group == group) {
        t->attr_idx = attr_idx;
        return DCF_OK;
    }
    free_attr(t);
    const size_t N = (size_t)t->g.N;
    const size_t n32 = 1 + 1 + (group == 1 ? 6 : 0);                                  // area, pending, bbox
    const size_t n64 = (group == 2 ? 3 : 0) + (group == 3 ? 5 : 0) + (group == 4 ? 14 : 0);
    const size_t bytes = (n32 * 4 + n64 * 8) * N + 256;
    CU(cudaMallocAsync(&t->attr_mem, bytes, ctx->stream));
    char *m = (char *)t->attr_mem;
    AttrBufs &a = t->attr;
    a.group = group;
    a.exact_g = t->dtype == U8 || t->dtype == U16;
    // 64-bit arrays first (alignment), then 32-bit
    auto take64 = [&]() { void *p = m; m += 8 * N; return p; };
    if (group == 2) for (int d = 0; d < 3; d++) a.s1[d] = (unsigned long long *)take64();
    if (group == 4) {
        for (int d = 0; d < 3; d++) a.s1[d] = (unsigned long long *)take64();
        for (int d = 0; d < 6; d++) a.s2[d] = (unsigned long long *)take64();
    }
    if (group == 3 || group == 4) for (int d = 0; d < 5; d++) a.gw[d] = take64();
    auto take32 = [&]() { void *p = m; m += 4 * N; return p; };
    a.area = (uint32_t *)take32();
    a.pending = (int *)take32();
    if (group == 1) {
        for (int d = 0; d < 3; d++) a.bmin[d] = (uint32_t *)take32();
        for (int d = 0; d < 3; d++) a.bmax[d] = (uint32_t *)take32();
    }
    // zero everything, then bbox minima to all-ones
    CU(cudaMemsetAsync(t->attr_mem, 0, (size_t)(m - (char *)t->attr_mem), ctx->stream));
    a.has_z = t->g.D > 1;
    if (group == 1) {
        CU(cudaMemsetAsync(a.bmin[0], 0xFF, (a.has_z ? 3 : 2) * 4 * N, ctx->stream));
        if (!a.has_z) launch_fill_u32((long long)N, a.bmax[2], 1u, ctx->sm_count, ctx->stream);
    }
    unsigned *count = ctx->d_err + 2;
    launch_attributes(view_of(t), a, count, ctx->up_steps, ctx->d_err, ctx->sm_count, ctx->stream);
    dcf_status st = check_launch(ctx, 4);
    if (st != DCF_OK) return st;
    unsigned R = 0;
    CU(cudaMemcpyAsync(&R, count, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    if (R > 0) {
        void *ws;
        st = scratch(ctx, 8, attr_rest_bytes(group, R), &ws);
        if (st != DCF_OK) return st;
        launch_attributes_rest(view_of(t), a, R, count, ws, ctx->d_err, ctx->sm_count, ctx->stream);
        st = check_launch(ctx, 4);
        if (st != DCF_OK) return st;
    }
    t->attr_idx = attr_idx;
    return DCF_OK;
}

dcf_status dcf_tree_build(dcf_ctx *ctx, const dcf_image *img, int attr_idx, dcf_tree **out)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !img || !out) return DCF_ERR_INVALID;
    *out = nullptr;
    if (!img->data) return set_err(ctx, DCF_ERR_INVALID, "null image data");
    if (img->dtype < DCF_U8 || img->dtype > DCF_F32) return set_err(ctx, DCF_ERR_INVALID, "bad dtype %d", img->dtype);
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES)
        return set_err(ctx, DCF_ERR_INVALID, "bad attribute %d", attr_idx);
    const uint64_t W = img->dims[0], H = img->dims[1], D = img->dims[2] ? img->dims[2] : 1;
    if (W == 0 || H == 0) return set_err(ctx, DCF_ERR_INVALID, "empty image");
    const unsigned long long N = W * H * D;
    if (W > 0x7FFFFFFF || H > 0x7FFFFFFF || D > 0x7FFFFFFF || N >= 0x7FFFFFFFull)
        return set_err(ctx, DCF_ERR_INVALID, "image too large (%llu pixels; limit 2^31-1)", N);
    int conn = img->connectivity;
    // io.c:64-79
    if (D > 1 && conn == 4) conn = 6;
    else if (conn == 8 && D > 1) conn = 26;
    else if (conn == 26 && D == 1) conn = 8;
    if (conn != 4 && conn != 6 && conn != 8 && conn != 26)
        return set_err(ctx, DCF_ERR_INVALID, "bad connectivity %d", img->connectivity);
    if (D == 1 && conn == 6) return set_err(ctx, DCF_ERR_INVALID, "connectivity 6 needs a 3-D image");
    for (int i = 0; i < 3; i++)
        if (!(img->pixdim[i] > 0.0f)) return set_err(ctx, DCF_ERR_INVALID, "pixdim must be positive");

    CU(cudaSetDevice(ctx->device));
    dcf_tree *t = new (std::nothrow) dcf_tree();
    if (!t) return DCF_ERR_NOMEM;
    t->ctx = ctx;
    t->stream = ctx->stream;
    t->g.W = (int)W;
    t->g.H = (int)H;
    t->g.D = (int)D;
    t->g.WH = (long long)W * H;
    t->g.N = (long long)N;
    t->g.conn = conn;
    t->g.level_sync = ctx->level_sync;
    if (D > 1) {
        t->g.tw = ctx->tile3d[0];
        t->g.th = ctx->tile3d[1];
        t->g.td = ctx->tile3d[2];
    } else {
        t->g.tw = ctx->tile2d[0];
        t->g.th = ctx->tile2d[1];
        t->g.td = 1;
    }
    t->dtype = img->dtype;
    t->tree_min = img->tree_type == DCF_MIN_TREE;
    for (int i = 0; i < 3; i++) t->pixdim[i] = img->pixdim[i];

    static const size_t esize[4] = {1, 2, 4, 4};
    const size_t in_bytes = N * esize[img->dtype];
    dcf_status st = DCF_OK;
    const void *d_in = img->data;
    void *tmp_in = nullptr;
#define TRY(call)                       \
    do {                                \
        cudaError_t _e = (call);        \
        if (_e != cudaSuccess) {        \
            st = set_err(ctx, _e == cudaErrorMemoryAllocation ? DCF_ERR_NOMEM : DCF_ERR_CUDA, "%s: %s", #call, \
                         cudaGetErrorString(_e)); \
            goto fail;                  \
        }                               \
    } while (0)
    TRY(cudaMallocAsync(&t->gval, N * sizeof(float), ctx->stream));
    TRY(cudaMallocAsync(&t->parent, N * sizeof(int), ctx->stream));
    TRY(cudaMallocAsync(&t->isroot, N, ctx->stream));
    TRY(cudaMallocAsync(&t->stats, 4 * sizeof(unsigned) + sizeof(unsigned long long), ctx->stream));
    t->num_nodes = (unsigned long long *)(t->stats + 4);
    if (!img->on_device) {
        TRY(cudaMallocAsync(&tmp_in, in_bytes, ctx->stream));
        TRY(cudaMemcpyAsync(tmp_in, img->data, in_bytes, cudaMemcpyHostToDevice, ctx->stream));
        d_in = tmp_in;
    }
    {
        unsigned init[4] = {0xFFFFFFFFu, 0u, 0u, 0u};
        TRY(cudaMemcpyAsync(t->stats, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
        TRY(cudaMemsetAsync(t->num_nodes, 0, sizeof(unsigned long long), ctx->stream));
        launch_stats(img->dtype, d_in, (long long)N, t->stats, t->stats + 1, t->stats + 2, ctx->sm_count,
                     ctx->stream);
        BuildArgs ba;
        ba.dtype = img->dtype;
        ba.tree_min = t->tree_min;
        ba.img = d_in;
        ba.g = t->g;
        ba.kmax = t->stats + 1;
        ba.gval = t->gval;
        void *nodes;
        st = scratch(ctx, 9, (size_t)N * 8, &nodes);
        if (st != DCF_OK) goto fail;
        ba.node = (unsigned long long *)nodes;
        ba.parent = t->parent;
        ba.isroot = t->isroot;
        ba.num_nodes = t->num_nodes;
        ba.err = ctx->d_err;
        ba.sm_count = ctx->sm_count;
        launch_build(ba, ctx->stream);
        st = check_launch(ctx, 4);
        if (st != DCF_OK) goto fail;
    }
    if (tmp_in) {
        // the stream orders the free after the kernels that read the input
        TRY(cudaFreeAsync(tmp_in, ctx->stream));
        tmp_in = nullptr;
    }
    st = compute_attributes(ctx, t, attr_idx);
    if (st != DCF_OK) goto fail;
    {
        std::lock_guard<std::mutex> lk(ctx->trees_mu);
        ctx->trees.insert(t);
    }
    *out = t;
    return DCF_OK;
fail:
    if (tmp_in) cudaFreeAsync(tmp_in, ctx->stream);
    dcf_tree_destroy(t);
    return st;
#undef TRY
}

dcf_status dcf_tree_set_attribute(dcf_ctx *ctx, dcf_tree *t, int attr_idx)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t) return DCF_ERR_INVALID;
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES) return set_err(ctx, DCF_ERR_INVALID, "bad attribute");
    return compute_attributes(ctx, t, attr_idx);
}

static dcf_status fetch_stats(dcf_ctx *ctx, dcf_tree *t, unsigned stats[3], unsigned long long *nodes)
{
    CU(cudaStreamSynchronize(ctx->stream));
    unsigned buf[4];
    CU(cudaMemcpy(buf, t->stats, sizeof(buf), cudaMemcpyDeviceToHost));
    if (nodes) CU(cudaMemcpy(nodes, t->num_nodes, sizeof(*nodes), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 3; i++) stats[i] = buf[i];
    return DCF_OK;
}

static float key_to_float_host(unsigned k)
{
    unsigned u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

dcf_status dcf_tree_info(const dcf_tree *tc, uint64_t *num_pixels, uint64_t *num_nodes, int *connectivity,
                         float *max_gval)
{
    if (!tc) return DCF_ERR_INVALID;
    dcf_tree *t = (dcf_tree *)tc;
    dcf_ctx *ctx = t->ctx;
    unsigned stats[3];
    unsigned long long nodes = 0;
    dcf_status st = fetch_stats(ctx, t, stats, &nodes);
    if (st != DCF_OK) return st;
    if (num_pixels) *num_pixels = (uint64_t)t->g.N;
    if (num_nodes) *num_nodes = nodes;
    if (connectivity) *connectivity = t->g.conn;
    if (max_gval) *max_gval = key_to_float_host(stats[1]);
    return DCF_OK;
}

// NaN inputs are detected by the statistics pass; report them at the first sync
static dcf_status check_nan(dcf_ctx *ctx, dcf_tree *t, float *gmax)
{
    unsigned stats[3];
    dcf_status st = fetch_stats(ctx, t, stats, nullptr);
    if (st != DCF_OK) return st;
    if (stats[2]) return set_err(ctx, DCF_ERR_NAN, "image holds %u NaN values", stats[2]);
    if (gmax) *gmax = key_to_float_host(stats[1]);
    return DCF_OK;
}

__global__ void k_widen(long long n, const int *__restrict__ in, long long *out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i];
}

dcf_status dcf_tree_parent(dcf_ctx *ctx, dcf_tree *t, int64_t *parent, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !parent) return DCF_ERR_INVALID;
    const size_t N = (size_t)t->g.N;
    long long *dst = (long long *)parent;
    if (!on_device) {
        void *s;
        dcf_status st = scratch(ctx, 0, N * 8, &s);
        if (st != DCF_OK) return st;
        dst = (long long *)s;
    }
    k_widen<<<grid_for(t->g.N, 256, ctx->sm_count), 256, 0, ctx->stream>>>(t->g.N, t->parent, dst);
    dcf_status st = check_launch(ctx, 1);
    if (st != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(parent, dst, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    st = sync_and_check(ctx);
    if (st != DCF_OK) return st;
    return check_nan(ctx, t, nullptr);
}

dcf_status dcf_tree_gval(dcf_ctx *ctx, dcf_tree *t, float *gval, int on_device)
{
    if (!ctx || !t || !gval) return DCF_ERR_INVALID;
    CU(cudaMemcpyAsync(gval, t->gval, (size_t)t->g.N * 4, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                       ctx->stream));
    dcf_status st = sync_and_check(ctx);
    if (st != DCF_OK) return st;
    return check_nan(ctx, t, nullptr);
}

static dcf_status check_attr(dcf_ctx *ctx, dcf_tree *t, int attr_idx)
{
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES) return set_err(ctx, DCF_ERR_INVALID, "bad attribute %d", attr_idx);
    if (!t->attr_mem) return set_err(ctx, DCF_ERR_STATE, "tree has no attributes");
    // attribute 0 (area) reads the area count every group's record carries
    if (attr_idx != 0 && ATTR_GROUP[attr_idx] != t->attr.group)
        return set_err(ctx, DCF_ERR_STATE, "attribute %d is not in the tree's group %d (use dcf_tree_set_attribute)",
                       attr_idx, t->attr.group);
    return DCF_OK;
}

dcf_status dcf_node_attribute(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int area, double *out, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !out) return DCF_ERR_INVALID;
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    const size_t N = (size_t)t->g.N;
    double *dst = out;
    if (!on_device) {
        void *s;
        st = scratch(ctx, 0, N * 8, &s);
        if (st != DCF_OK) return st;
        dst = (double *)s;
    }
    launch_node_attr(view_of(t), t->attr, attr_idx, area != 0, dst, ctx->sm_count, ctx->stream);
    st = check_launch(ctx, 1);
    if (st != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(out, dst, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    st = sync_and_check(ctx);
    if (st != DCF_OK) return st;
    return check_nan(ctx, t, nullptr);
}

// longest possible root path: every node on it has a distinct grey level
static long long depth_bound(const dcf_tree *t)
{
    if (t->dtype == U8) return 256;
    if (t->dtype == U16) return 65536;
    return t->g.N;
}

static dcf_status run_filter(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int rule, double lambda, int extract,
                             float *dst)
{
    const size_t N = (size_t)t->g.N;
    FilterWork w{};
    void *p;
    dcf_status st;
    if ((st = scratch(ctx, 1, N, &p)) != DCF_OK) return st;
    w.flag = (unsigned char *)p;
    if ((st = scratch(ctx, 2, N * 4, &p)) != DCF_OK) return st;
    w.target = (int *)p;
    if (rule == 2) {
        if ((st = scratch(ctx, 3, N * 4, &p)) != DCF_OK) return st;
        w.kept = (unsigned *)p;
    }
    if (rule == 1 || rule == 3) {
        if ((st = scratch(ctx, 3, N * 4, &p)) != DCF_OK) return st;
        w.jump = (int *)p;
        if ((st = scratch(ctx, 4, N * 4, &p)) != DCF_OK) return st;
        w.jump2 = (int *)p;
        w.best2 = (int *)p;
        if (rule == 3) {
            if ((st = scratch(ctx, 5, N * 8, &p)) != DCF_OK) return st;
            w.acc = (double *)p;
            if ((st = scratch(ctx, 6, N * 8, &p)) != DCF_OK) return st;
            w.acc2 = (double *)p;
            w.remaining = ctx->d_err + 1;
        } else {
            if ((st = scratch(ctx, 5, N * 4, &p)) != DCF_OK) return st;
            w.best2 = (int *)p;
        }
    }
    TreeView v = view_of(t);
    launch_filter(v, t->attr, attr_idx, rule, lambda, extract != 0, dst, w, depth_bound(t), ctx->d_err,
                  ctx->sm_count, ctx->stream);
    return check_launch(ctx, 3);
}

dcf_status dcf_filter(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int rule, double lambda, int extract, float *out,
                      int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !out) return DCF_ERR_INVALID;
    if (rule < 0 || rule > 3) return set_err(ctx, DCF_ERR_INVALID, "bad rule %d", rule);
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    const size_t N = (size_t)t->g.N;
    float *dst = out;
    if (!on_device) {
        void *s;
        if ((st = scratch(ctx, 7, N * 4, &s)) != DCF_OK) return st;
        dst = (float *)s;
    }
    st = run_filter(ctx, t, attr_idx, rule, lambda, extract, dst);
    if (st != DCF_OK) return st;
    if (!on_device) {
        CU(cudaMemcpyAsync(out, dst, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
        st = sync_and_check(ctx);
        if (st != DCF_OK) return st;
        return check_nan(ctx, t, nullptr);
    }
    return DCF_OK;
}

dcf_status dcf_dmp(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int rule, const float *lvec, int num_lambdas, float *out,
                   int on_device)
{
    if (!ctx || !t || !out || !lvec || num_lambdas < 1) return DCF_ERR_INVALID;
    const size_t N = (size_t)t->g.N;
    for (int i = 0; i + 1 < num_lambdas; i++) {
        // operation.c:63-76: filter at lvec[i+1] (as float), then gval - filtered
        dcf_status st = dcf_filter(ctx, t, attr_idx, rule, (double)lvec[i + 1], 1, out + (size_t)i * N, on_device);
        if (st != DCF_OK) return st;
    }
    return DCF_OK;
}

dcf_status dcf_attribute_check(dcf_ctx *ctx, dcf_tree *t, int attr_idx, float *out, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !out) return DCF_ERR_INVALID;
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    const size_t N = (size_t)t->g.N;
    float *dst = out;
    if (!on_device) {
        void *s;
        if ((st = scratch(ctx, 7, N * 4, &s)) != DCF_OK) return st;
        dst = (float *)s;
    }
    launch_check(view_of(t), t->attr, attr_idx, dst, ctx->sm_count, ctx->stream);
    st = check_launch(ctx, 1);
    if (st != DCF_OK) return st;
    if (!on_device) {
        CU(cudaMemcpyAsync(out, dst, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
        st = sync_and_check(ctx);
        if (st != DCF_OK) return st;
        return check_nan(ctx, t, nullptr);
    }
    return DCF_OK;
}

static dcf_status spectrum_common(dcf_ctx *ctx, dcf_tree *t, int a1, const float *l1, int n1, int a2,
                                  const float *l2, int n2, double *spec, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (n1 < 1 || n2 < 1 || !l1 || !l2 || !spec) return set_err(ctx, DCF_ERR_INVALID, "bad lambda vectors");
    const size_t nb = (size_t)n1 * n2;
    void *s;
    dcf_status st;
    // lambda vectors and (for host output) the spectrum live in one scratch block
    const size_t lbytes = ((size_t)(n1 + n2) * 4 + 255) / 256 * 256;
    if ((st = scratch(ctx, 0, lbytes + nb * 8, &s)) != DCF_OK) return st;
    float *dl = (float *)s;
    double *dspec = on_device ? spec : (double *)((char *)s + lbytes);
    CU(cudaMemcpyAsync(dl, l1, (size_t)n1 * 4, cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaMemcpyAsync(dl + n1, l2, (size_t)n2 * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (!on_device) CU(cudaMemcpyAsync(dspec, spec, nb * 8, cudaMemcpyHostToDevice, ctx->stream));
    launch_spectrum(view_of(t), t->attr, a1, dl, n1, a2, dl + n1, n2, dspec, ctx->sm_count, ctx->stream);
    st = check_launch(ctx, 1);
    if (st != DCF_OK) return st;
    if (!on_device) {
        CU(cudaMemcpyAsync(spec, dspec, nb * 8, cudaMemcpyDeviceToHost, ctx->stream));
        st = sync_and_check(ctx);
        if (st != DCF_OK) return st;
        return check_nan(ctx, t, nullptr);
    }
    return DCF_OK;
}

dcf_status dcf_pattern_spectrum(dcf_ctx *ctx, dcf_tree *t, int attr_idx, const float *lvec, int num_lambdas,
                                double *spectrum, int on_device)
{
    if (!ctx || !t) return DCF_ERR_INVALID;
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    static const float one = 0.0f;
    return spectrum_common(ctx, t, attr_idx, lvec, num_lambdas, 0, &one, 1, spectrum, on_device);
}

dcf_status dcf_pattern_spectrum2d(dcf_ctx *ctx, dcf_tree *t, int attr1, const float *lvec1, int n1, int attr2,
                                  const float *lvec2, int n2, double *spectrum, int on_device)
{
    if (!ctx || !t) return DCF_ERR_INVALID;
    // operation.c:93-100
    if (attr1 == 0 && attr2 != 0)
        return set_err(ctx, DCF_ERR_INVALID, "the attribute with the highest index must come first");
    dcf_status st = check_attr(ctx, t, attr1);
    if (st != DCF_OK) return st;
    if (attr2 != 0) {
        if (attr2 < 0 || attr2 >= DCF_NUM_ATTRIBUTES || ATTR_GROUP[attr2] != t->attr.group)
            return set_err(ctx, DCF_ERR_INVALID, "both 2-D spectrum attributes must be in one group");
    }
    return spectrum_common(ctx, t, attr1, lvec1, n1, attr2 == 0 ? -1 : attr2, lvec2, n2, spectrum, on_device);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free direct-rule filter.
//
// Some callers cannot allocate device memory at the moment they filter: a host
// framework whose caching allocator has already reserved the device's free memory,
// or a real-time loop that must never wait on, or fail in, an allocation.  For them
// the per-pixel scratch of the direct rule (one survive byte and one resolved-node
// index per pixel) lives in this fixed device array instead of the context's
// buffers.  The array is NOALLOC_MAX_PIXELS * 5 bytes (40 MiB) and every GPU that
// loads the library keeps it until the process exits.
// ---------------------------------------------------------------------------
static constexpr long long NOALLOC_MAX_PIXELS = 1LL << 23;  // 8,388,608 pixels
static constexpr size_t NOALLOC_BYTES = (size_t)NOALLOC_MAX_PIXELS * 5 + 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64];  // device address of g_noalloc_scratch, per device

extern "C" dcf_status dcf_filter_direct_noalloc(dcf_ctx *ctx, dcf_tree *t, int attr_idx, double lambda,
                                                int extract, float *out_device)
{
    if (!ctx || !t || !out_device) return DCF_ERR_INVALID;
    if (t->g.N > NOALLOC_MAX_PIXELS)
        return set_err(ctx, DCF_ERR_INVALID, "dcf_filter_direct_noalloc: %lld pixels exceed the fixed scratch of %lld",
                       (long long)t->g.N, NOALLOC_MAX_PIXELS);
    if (ctx->device < 0 || ctx->device >= 64) return set_err(ctx, DCF_ERR_INVALID, "device index out of range");
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    void *base = nullptr;
    {
        // one-time set-up per device, with that device current: the host-side
        // name g_noalloc_scratch is not a device address, so look the address up
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[ctx->device]) {
            CU(cudaSetDevice(ctx->device));
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p)
                return set_err(ctx, DCF_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
            g_noalloc_ptr[ctx->device] = p;
        }
        base = g_noalloc_ptr[ctx->device];
    }
    ActiveScope active_scope_(ctx);
    // layout: N resolved-node indices (int32), then N survive bytes; every call
    // rewrites both for all pixels (k_flag resets the indices), so nothing carries
    // over from the previous call
    FilterWork w{};
    w.target = (int *)base;
    w.flag = (unsigned char *)base + (size_t)NOALLOC_MAX_PIXELS * 4;
    launch_filter(view_of(t), t->attr, attr_idx, 0, lambda, extract != 0, out_device, w, depth_bound(t), ctx->d_err,
                  ctx->sm_count, ctx->stream);
    return check_launch(ctx, 3);
}
