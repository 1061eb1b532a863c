// C-ABI entry points (include/dcf.h).  Every call validates its arguments on the
// host, enqueues kernels on the context's stream and only synchronises when it
// must hand data back to host memory; device-side failures (loop bounds) are
// collected in a device error word and reported by the next synchronising call.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <vector>

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
    // build tile of 2-D images (width, height): 128 x 32 builds faster than 64 x 64
    // (fewer band-merge levels) at the price of more seam edges
    int tile2d[2] = {128, 32};
    int tile3d[3] = {16, 16, 16};     // build tile of 3-D images
    int level_sync = 1;               // barrier between band-merge levels inside a tile
    // level buckets of the seam merge: 1 = every cross-tile edge at once, from a
    // compacted list (full warps: most face/offset work items hold no edge); 0 = at
    // once straight from the work items
    int seam_buckets = 1;
    // Test knobs, read from the environment at creation.  merge_bound (DCF_MERGE_BOUND):
    // iteration limit of every tree-merge loop (0 = the built-in limits); a small
    // value makes merges give up, which must surface as DCF_ERR_TIMEOUT.
    // fail_alloc (DCF_FAIL_ALLOC = k): the k-th device allocation made through this
    // context (counting from 0) reports out-of-memory without allocating, which must
    // surface as DCF_ERR_NOMEM with nothing leaked; -1 = off.
    long long merge_bound = 0;
    long long fail_alloc = -1;
    long long allocs = 0;
    std::mutex trees_mu;
    std::set<dcf_tree *> trees;       // live trees; orphaned (stream cleared) when the context goes
    DevBuf scratch[16];               // reusable work buffers (filter, spectra, attributes, seams)
    DevBuf stage;                     // the image staged by dcf_image_stage (stream-ordered pool memory)
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
void note_launch()
{
    if (t_active) t_active->launches++;
}
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
    int *nodes = nullptr;                    // level roots in ascending order (node_list_bytes)
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

// Every device allocation of the library goes through these two, so that the
// allocation-failure knob (dcf_ctx::fail_alloc) reaches each of them.
static bool alloc_refused(dcf_ctx *c)
{
    if (!c) return false;
    return c->allocs++ == c->fail_alloc;
}
template <typename T>
static cudaError_t dmalloc(dcf_ctx *c, T **p, size_t bytes)
{
    if (alloc_refused(c)) return cudaErrorMemoryAllocation;
    return cudaMalloc((void **)p, bytes);
}
template <typename T>
static cudaError_t dmalloc_async(dcf_ctx *c, T **p, size_t bytes, cudaStream_t s)
{
    if (alloc_refused(c)) return cudaErrorMemoryAllocation;
    return cudaMallocAsync((void **)p, bytes, s);
}

#define CU(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t _e = (call);                                                                          \
        if (_e != cudaSuccess) return set_err(ctx, _e == cudaErrorMemoryAllocation ? DCF_ERR_NOMEM : DCF_ERR_CUDA, \
                                              "%s: %s", #call, cudaGetErrorString(_e));                  \
    } while (0)

static dcf_status check_launch(dcf_ctx *ctx, int)
{
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
        CU(dmalloc(ctx, &b.p, bytes));
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
        if (sscanf(e, "%dx%d", &a, &b) == 2 && a > 0 && b > 0 && a * b <= TILE_MAX_PIX &&
            tile_smem_bytes(a, b, 1) <= 48 * 1024) {
            ctx->tile2d[0] = a;
            ctx->tile2d[1] = b;
        }
    }
    if (const char *e = getenv("DCF_LEVEL_SYNC")) ctx->level_sync = atoi(e) != 0;
    if (const char *e = getenv("DCF_SEAM_BUCKETS")) {
        int v = atoi(e);
        if (v >= 0 && v <= 1024) ctx->seam_buckets = v;
    }
    if (const char *e = getenv("DCF_MERGE_BOUND")) {
        long long v = atoll(e);
        if (v > 0) ctx->merge_bound = v;
    }
    if (const char *e = getenv("DCF_FAIL_ALLOC")) ctx->fail_alloc = atoll(e);
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
    if (ctx->stage.p) cudaFreeAsync(ctx->stage.p, ctx->stream);
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

void *dcf_ctx_stream(const dcf_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

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
    dev_free(t->nodes, t->stream);
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
    v.nodes = t->nodes;
    v.num_nodes = t->num_nodes;
    for (int i = 0; i < 3; i++) v.pixdim[i] = t->pixdim[i];
    v.integer_levels = t->dtype == U8 || t->dtype == U16;
    return v;
}

// Record arrays of an attribute group over N pixels, carved from one allocation:
// 64-bit arrays first (alignment), then 32-bit ones.
static size_t attr_bytes(int group, size_t N)
{
    const size_t n32 = 1 + 1 + (group == 1 ? 6 : 0);                                  // area, pending, bbox
    const size_t n64 = (group == 2 ? 3 : 0) + (group == 3 ? 5 : 0) + (group == 4 ? 14 : 0);
    return (n32 * 4 + n64 * 8 + 1) * N + 256;  // + one `single` byte per pixel
}

static void attr_carve(AttrBufs &a, int group, bool exact_g, bool has_z, size_t N, void *mem)
{
    char *m = (char *)mem;
    a = AttrBufs();
    a.group = group;
    a.exact_g = exact_g;
    a.has_z = has_z;
    a.grey = group == 3;  // the inertia group adds them only on request (compute_attributes)
    auto take64 = [&]() { void *p = m; m += 8 * N; return p; };
    if (group == 2) for (int d = 0; d < 3; d++) a.s1[d] = (unsigned long long *)take64();
    if (group == 4) {
        for (int d = 0; d < 3; d++) a.s1[d] = (unsigned long long *)take64();
        for (int d = 0; d < 6; d++) a.s2[d] = (unsigned long long *)take64();
    }
    if (group == 3 || group == 4) for (int d = 0; d < 5; d++) a.gw[d] = take64();
    // the 32-bit fields interleaved per node (Field): the extent group's record is
    // area, pending, bmin x/y/z, bmax x/y/z; the other groups pair area and pending
    const int words = group == 1 ? REC1_WORDS : 2;
    uint32_t *rec = (uint32_t *)m;
    m += 4 * (size_t)words * N;
    a.area = Field<uint32_t>{rec, words};
    a.pending = Field<int>{(int *)rec + 1, words};
    if (group == 1)
        for (int d = 0; d < 3; d++) {
            a.bmin[d] = Field<uint32_t>{rec + 2 + d, words};
            a.bmax[d] = Field<uint32_t>{rec + 5 + d, words};
        }
    a.single = (unsigned char *)m;
}

// start values of the level roots' records (the only records any pass reads)
static cudaError_t attr_zero(const AttrBufs &a, const int *nodes, const unsigned long long *num_nodes, size_t N,
                             int sm, cudaStream_t s)
{
    launch_attr_init(a, NodeSet{nodes, num_nodes}, (long long)N, sm, s);
    return cudaGetLastError();
}

// allocate and accumulate the records of attr_idx's group
// need_grey: the inertia group must also accumulate the grey-weighted sums (the
// tree file's weighted centroids); its attributes 13-17 do not read them
static dcf_status compute_attributes(dcf_ctx *ctx, dcf_tree *t, int attr_idx, bool need_grey = false)
{
    const int group = ATTR_GROUP[attr_idx];
    if (t->attr_mem && t->attr.group == group && (!need_grey || t->attr.grey)) {
        t->attr_idx = attr_idx;
        return DCF_OK;
    }
    free_attr(t);
    const size_t N = (size_t)t->g.N;
    CU(dmalloc_async(ctx, &t->attr_mem, attr_bytes(group, N), ctx->stream));
    AttrBufs &a = t->attr;
    attr_carve(a, group, t->dtype == U8 || t->dtype == U16, t->g.D > 1, N, t->attr_mem);
    if (need_grey) a.grey = true;
    CU(attr_zero(a, t->nodes, t->num_nodes, N, ctx->sm_count, ctx->stream));
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
    // each extent below 2^31, so W * H and then (W * H) * D cannot wrap around 64 bits
    if (W > 0x7FFFFFFF || H > 0x7FFFFFFF || D > 0x7FFFFFFF || W * H >= 0x7FFFFFFFull ||
        W * H * D >= 0x7FFFFFFFull)
        return set_err(ctx, DCF_ERR_INVALID, "image too large (%llu x %llu x %llu; limit 2^31-1 pixels)",
                       (unsigned long long)W, (unsigned long long)H, (unsigned long long)D);
    const unsigned long long N = W * H * D;
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
    t->g.merge_bound = ctx->merge_bound;
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
    TRY(dmalloc_async(ctx, &t->gval, N * sizeof(float), ctx->stream));
    TRY(dmalloc_async(ctx, &t->parent, N * sizeof(int), ctx->stream));
    TRY(dmalloc_async(ctx, &t->isroot, N, ctx->stream));
    TRY(dmalloc_async(ctx, &t->nodes, node_list_bytes((long long)N), ctx->stream));
    TRY(dmalloc_async(ctx, &t->stats, 4 * sizeof(unsigned) + sizeof(unsigned long long), ctx->stream));
    t->num_nodes = (unsigned long long *)(t->stats + 4);
    if (!img->on_device) {
        TRY(dmalloc_async(ctx, &tmp_in, in_bytes, ctx->stream));
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
        ba.nodes = t->nodes;
        ba.num_nodes = t->num_nodes;
        ba.err = ctx->d_err;
        ba.sm_count = ctx->sm_count;
        if (ctx->seam_buckets > 0) {
            const long long ntiles = (long long)((W + t->g.tw - 1) / t->g.tw) * ((H + t->g.th - 1) / t->g.th) *
                                     ((D + t->g.td - 1) / t->g.td);
            const long long cap = seam_edge_bound(t->g, ntiles);
            void *sm;
            st = scratch(ctx, 12, seam_edges_bytes(cap, ctx->seam_buckets), &sm);
            if (st != DCF_OK) goto fail;
            ba.seam = seam_edges_carve(sm, cap, ctx->seam_buckets);
        }
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
    k_widen<<<grid_for(t->g.N, 256, ctx->sm_count), 256, 0, ctx->stream>>>(t->g.N, t->parent, dst); note_launch();
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

dcf_status dcf_csl(dcf_ctx *ctx, dcf_tree *t, int attr_idx, const float *lvec, int num_lambdas, float *contrast,
                   float *scale, float *luminance, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !lvec || num_lambdas < 1 || !contrast || !scale || !luminance) return DCF_ERR_INVALID;
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    const size_t N = (size_t)t->g.N;
    const size_t lbytes = ((size_t)num_lambdas * 4 + 255) / 256 * 256;
    void *work, *io;
    if ((st = scratch(ctx, 13, csl_work_bytes((long long)N) + lbytes, &work)) != DCF_OK) return st;
    float *dl = (float *)((char *)work + csl_work_bytes((long long)N));
    CU(cudaMemcpyAsync(dl, lvec, (size_t)num_lambdas * 4, cudaMemcpyHostToDevice, ctx->stream));
    float *out[3] = {contrast, scale, luminance};
    if (!on_device) {
        if ((st = scratch(ctx, 7, N * 12, &io)) != DCF_OK) return st;
        for (int i = 0; i < 3; i++) out[i] = (float *)io + i * N;
    }
    launch_csl(view_of(t), t->attr, attr_idx, dl, num_lambdas, out[0], out[1], out[2], work, ctx->d_err + 1,
               ctx->sm_count, ctx->stream);
    if ((st = check_launch(ctx, 0)) != DCF_OK) return st;
    if (!on_device) {
        CU(cudaMemcpyAsync(contrast, out[0], N * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaMemcpyAsync(scale, out[1], N * 4, cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaMemcpyAsync(luminance, out[2], N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    st = sync_and_check(ctx);
    if (st != DCF_OK) return st;
    return check_nan(ctx, t, nullptr);
}

// readout of attribute (or tree-file column) `code` into host memory
static dcf_status readout_host(dcf_ctx *ctx, dcf_tree *t, int code, bool area, std::vector<double> &out)
{
    const size_t N = (size_t)t->g.N;
    void *s;
    dcf_status st = scratch(ctx, 0, N * 8, &s);
    if (st != DCF_OK) return st;
    launch_node_attr(view_of(t), t->attr, code, area, (double *)s, ctx->sm_count, ctx->stream);
    if ((st = check_launch(ctx, 1)) != DCF_OK) return st;
    out.resize(N);
    CU(cudaMemcpyAsync(out.data(), s, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

dcf_status dcf_tree_export(dcf_ctx *ctx, dcf_tree *t, int attr_idx, const char *path)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !path) return DCF_ERR_INVALID;
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES) return set_err(ctx, DCF_ERR_INVALID, "bad attribute %d", attr_idx);
    if (!t->attr_mem || ATTR_GROUP[attr_idx] != t->attr.group)
        return set_err(ctx, DCF_ERR_STATE, "attribute %d is not in the tree's group (use dcf_tree_set_attribute)",
                       attr_idx);
    const int group = ATTR_GROUP[attr_idx];
    dcf_status st;
    if (group == 4 && (st = compute_attributes(ctx, t, attr_idx, true)) != DCF_OK) return st;
    const size_t N = (size_t)t->g.N;
    std::vector<int64_t> par(N);
    std::vector<float> gv(N);
    if ((st = dcf_tree_parent(ctx, t, par.data(), 0)) != DCF_OK) return st;
    if ((st = dcf_tree_gval(ctx, t, gv.data(), 0)) != DCF_OK) return st;
    std::vector<double> area;
    if ((st = readout_host(ctx, t, attr_idx, true, area)) != DCF_OK) return st;
    // the group's extra columns (io.c:1454-1462 header, :1518-1547 rows)
    static const int g1[] = {1, 2, 3, 4, 5}, g2[] = {6, 7, 8}, g3[] = {9, 10, 11},
                     g4[] = {INERTIA_COL0, INERTIA_COL0 + 1, INERTIA_COL0 + 2, INERTIA_COL0 + 3, INERTIA_COL0 + 4,
                             INERTIA_COL0 + 5, 14, 15, 16, 17};
    const int *codes = group == 1 ? g1 : group == 2 ? g2 : group == 3 ? g3 : g4;
    const int ncol = group == 0 ? 0 : group == 1 ? 5 : (group == 4 ? 10 : 3);
    std::vector<std::vector<double>> cols(ncol);
    for (int c = 0; c < ncol; c++)
        if ((st = readout_host(ctx, t, codes[c], false, cols[c])) != DCF_OK) return st;
    FILE *f = fopen(path, "w");
    if (!f) return set_err(ctx, DCF_ERR_IO, "cannot open %s for writing", path);
    fprintf(f, "index,x,y,z,gval,parent,flux,area,");
    if (group == 1) fprintf(f, "area_enc_rect,diag_enc_rect,x_extent,y_extent,z_extent");
    else if (group == 2) fprintf(f, "x_mean,y_mean,z_mean");
    else if (group == 3) fprintf(f, "x_wmean,y_wmean,z_wmean");
    else if (group == 4) fprintf(f, "x_mean,y_mean,z_mean,x_wmean,y_wmean,z_wmean,elong,flat,spars,ncomp");
    fprintf(f, "\n");
    const uint64_t W = (uint64_t)t->g.W, WH = (uint64_t)t->g.WH;
    for (size_t i = 0; i < N; i++) {
        const int64_t q = par[i];
        if (q >= 0 && gv[q] == gv[i]) continue;  // not a level root (flood.h:29-32)
        const long x = (long)((i % WH) % W), y = (long)((i % WH) / W), z = (long)(i / WH);
        const long size = (long)area[i];
        const float dh = q >= 0 ? gv[i] - gv[q] : gv[i];
        fprintf(f, "%ld,%ld,%ld,%ld,%f,%ld,%f,%ld,", (long)i, x, y, z, (double)gv[i], (long)q,
                (double)(dh * (float)size), size);
        if (group == 1 || group == 2 || group == 3) {
            for (int c = 0; c < ncol; c++) fprintf(f, c ? ",%.2f" : "%.2f", (double)(float)cols[c][i]);
        } else if (group == 4) {
            for (int c = 0; c < 6; c++) fprintf(f, "%.2f,", (double)(float)cols[c][i]);
            fprintf(f, "%.3f,%.3f,%.3f,%.4f ", (double)(float)cols[6][i], (double)(float)cols[7][i],
                    (double)(float)cols[8][i], (double)(float)cols[9][i]);
        }
        fprintf(f, "\n");
    }
    if (fclose(f) != 0) return set_err(ctx, DCF_ERR_IO, "write to %s failed", path);
    return DCF_OK;
}

// longest possible root path: every node on it has a distinct grey level
static long long depth_bound(const dcf_tree *t)
{
    if (t->dtype == U8) return 256;
    if (t->dtype == U16) return 65536;
    return t->g.N;
}

static dcf_status run_filter(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int rule, double lambda, int extract,
                             void *dst, int out_dtype = F32)
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
                  ctx->sm_count, ctx->stream, out_dtype);
    return check_launch(ctx, 3);
}

dcf_status dcf_filter_as(dcf_ctx *ctx, dcf_tree *t, int attr_idx, int rule, double lambda, int extract,
                         int out_dtype, void *out, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !out) return DCF_ERR_INVALID;
    if (rule < 0 || rule > 3) return set_err(ctx, DCF_ERR_INVALID, "bad rule %d", rule);
    if (out_dtype != DCF_F32 && !((out_dtype == DCF_U8 || out_dtype == DCF_U16) && out_dtype == t->dtype))
        return set_err(ctx, DCF_ERR_INVALID, "output type %d: float, or the input's own u8/u16 type", out_dtype);
    dcf_status st = check_attr(ctx, t, attr_idx);
    if (st != DCF_OK) return st;
    static const size_t esize[4] = {1, 2, 4, 4};
    const size_t bytes = (size_t)t->g.N * esize[out_dtype];
    void *dst = out;
    if (!on_device && (st = scratch(ctx, 7, bytes, &dst)) != DCF_OK) return st;
    if ((st = run_filter(ctx, t, attr_idx, rule, lambda, extract, dst, out_dtype)) != DCF_OK) return st;
    if (!on_device) {
        CU(cudaMemcpyAsync(out, dst, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        if ((st = sync_and_check(ctx)) != DCF_OK) return st;
        return check_nan(ctx, t, nullptr);
    }
    return DCF_OK;
}

dcf_status dcf_image_stage(dcf_ctx *ctx, const dcf_image *in, dcf_image *out)
{
    if (!ctx || !in || !out || !in->data) return DCF_ERR_INVALID;
    if (in->dtype < DCF_U8 || in->dtype > DCF_F32) return set_err(ctx, DCF_ERR_INVALID, "bad dtype %d", in->dtype);
    *out = *in;
    if (in->on_device) return DCF_OK;
    const uint64_t D = in->dims[2] ? in->dims[2] : 1;
    if (in->dims[0] > 0x7FFFFFFF || in->dims[1] > 0x7FFFFFFF || D > 0x7FFFFFFF ||
        in->dims[0] * in->dims[1] >= 0x7FFFFFFFull || in->dims[0] * in->dims[1] * D >= 0x7FFFFFFFull)
        return set_err(ctx, DCF_ERR_INVALID, "image too large");
    static const size_t esize[4] = {1, 2, 4, 4};
    const size_t bytes = (size_t)(in->dims[0] * in->dims[1] * D) * esize[in->dtype];
    CU(cudaSetDevice(ctx->device));
    DevBuf &b = ctx->stage;
    if (b.bytes < bytes) {
        // earlier builds may still read the old buffer: free it in stream order
        if (b.p) CU(cudaFreeAsync(b.p, ctx->stream));
        b.p = nullptr;
        b.bytes = 0;
        CU(dmalloc_async(ctx, &b.p, bytes, ctx->stream));
        b.bytes = bytes;
    }
    CU(cudaMemcpyAsync(b.p, in->data, bytes, cudaMemcpyHostToDevice, ctx->stream));
    out->data = b.p;
    out->on_device = 1;
    return DCF_OK;
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
    // the fixed array belongs to one device: a tree of another context's device
    // would be filtered in the wrong device's memory
    if (!t->ctx || t->ctx->device != ctx->device)
        return set_err(ctx, DCF_ERR_INVALID, "dcf_filter_direct_noalloc: tree was built on another device");
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
            // the caller's current device is put back afterwards
            int prev = -1;
            CU(cudaGetDevice(&prev));
            CU(cudaSetDevice(ctx->device));
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            cudaSetDevice(prev);
            if (e != cudaSuccess || !p)
                return set_err(ctx, DCF_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s", cudaGetErrorString(e));
            g_noalloc_ptr[ctx->device] = p;
        }
        base = g_noalloc_ptr[ctx->device];
    }
    ActiveScope active_scope_(ctx);
    // layout: N resolved-node indices (int32), then N survive bytes; every call
    // rewrites both at every level root of the tree (k_flag resets the indices),
    // the only entries the filter passes read, so nothing carries over from the
    // previous call
    FilterWork w{};
    w.target = (int *)base;
    w.flag = (unsigned char *)base + (size_t)NOALLOC_MAX_PIXELS * 4;
    launch_filter(view_of(t), t->attr, attr_idx, 0, lambda, extract != 0, out_device, w, depth_bound(t), ctx->d_err,
                  ctx->sm_count, ctx->stream);
    return check_launch(ctx, 3);
}

// ---------------------------------------------------------------------------
// Batches of 2-D cutouts and the adjoint (no reference counterpart).
//
// A batch owns every device buffer its runs need, allocated once at creation (or
// on the first run that needs it), so a run issues no allocation and can be
// recorded as one CUDA graph: statistics, persistent tile build, seam merge,
// canonical form, attribute pass, filter and spectra.  The only step that would
// need the host in the middle is the attribute pass's pointer-jumping phase,
// whose scratch is sized by the number of nodes left after the bounded
// bottom-up fold; a graph run uses a fixed capacity learned on the first
// (ungraphed) run, and a run whose count exceeds it is detected after the graph,
// redone ungraphed and the capacity doubled.
// ---------------------------------------------------------------------------
struct BatchKey {
    const void *pixels = nullptr;
    float *filtered = nullptr;
    double *spectra = nullptr;
    int filter_attr = -1, a1 = -1, a2 = -1, n1 = 0, n2 = 0;
    double lambda = 0.0;
    int tw = 0, th = 0, ctas = 0, chunk = 0;
    unsigned cap = 0;
    void *rest_mem = nullptr;
    bool operator==(const BatchKey &o) const
    {
        return pixels == o.pixels && filtered == o.filtered && spectra == o.spectra && filter_attr == o.filter_attr &&
               a1 == o.a1 && a2 == o.a2 && n1 == o.n1 && n2 == o.n2 && lambda == o.lambda && tw == o.tw &&
               th == o.th && ctas == o.ctas && chunk == o.chunk && cap == o.cap && rest_mem == o.rest_mem;
    }
};

struct dcf_batch {
    dcf_ctx *ctx = nullptr;
    int count = 0, dtype = F32, conn = 8, group = 0, attr_idx = 0;
    float pixdim[3] = {1, 1, 1};
    long long N = 0;
    std::vector<BatchImg> imgs;
    BatchImg *d_imgs = nullptr;
    long long *d_offs = nullptr;
    // schedule: tile shape, CTAs per SM of the persistent kernel, tiles per queue grab
    int tw = 64, th = 64, ctas = 1, chunk = 1;
    int seam_buckets = 16;                   // level buckets of the seam merge (0: all edges at once)
    int up_steps = 2048;                     // bottom-up fold steps per walker
    long long merge_bound = 0;               // the context's merge-loop limit (test knob)
    int ntiles = 0;
    size_t tiles_cap = 0;
    BatchTile *d_tiles = nullptr;
    unsigned *d_misc = nullptr;              // [0] queue counter [1] rest count [2] kmin [3] kmax [4] nans
    unsigned long long *d_nodes = nullptr;   // node count of the last build
    void *pixels = nullptr;                  // input copy for host-side pixels
    float *gval = nullptr;
    unsigned long long *node = nullptr;
    int *parent = nullptr;
    unsigned char *isroot = nullptr;
    int *nodes = nullptr;                    // level roots in ascending order (node_list_bytes)
    void *attr_mem = nullptr;
    AttrBufs attr;
    void *seam_mem = nullptr;                // level-ordered seam merge scratch
    size_t seam_bytes = 0;
    SeamEdges seam;
    unsigned rest_cap = 0;                   // graph runs: pointer-jumping capacity (0: not learned yet)
    size_t rest_bytes = 0;
    void *rest_mem = nullptr;
    unsigned char *flag = nullptr;
    int *target = nullptr;
    float *filtered = nullptr;               // host-output staging
    double *spectra = nullptr;
    size_t spectra_cap = 0;
    float *lvec = nullptr;                   // device lambda vectors (lvec1 then lvec2)
    size_t lvec_cap = 0;
    double *adj_acc = nullptr;
    float *adj_io = nullptr;                 // host-side adjoint staging: v, then grad
    double *adj_w = nullptr;
    size_t adj_w_cap = 0;
    // last run
    bool valid = false;
    dcf_op_set ops{};
    // recorded graphs, one per distinct run configuration (a forward with outputs
    // and a recomputation without them alternate in training), least recently used
    // dropped beyond MAX_GRAPHS
    struct Graph {
        BatchKey key;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        uint64_t kernels = 0, used = 0;
    };
    static constexpr size_t MAX_GRAPHS = 4;
    std::vector<Graph> graphs;
    uint64_t uses = 0;
    uint64_t graph_kernels = 0;              // kernel nodes of the last graph launched
};

static void batch_drop_graph(dcf_batch *b)
{
    for (auto &g : b->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
    }
    b->graphs.clear();
}

static TreeView batch_view(const dcf_batch *b)
{
    TreeView v;
    v.g = Geom{};
    v.g.W = (int)b->N;  // unused by the node-parallel passes
    v.g.H = v.g.D = 1;
    v.g.WH = v.g.N = b->N;
    v.g.conn = b->conn;
    v.g.tw = b->tw;
    v.g.th = b->th;
    v.g.td = 1;
    v.g.level_sync = 1;
    v.g.merge_bound = b->merge_bound;
    v.tree_min = false;
    v.kmax = b->d_misc + 3;
    v.gval = b->gval;
    v.parent = b->parent;
    v.isroot = b->isroot;
    v.nodes = b->nodes;
    v.num_nodes = b->d_nodes;
    for (int i = 0; i < 3; i++) v.pixdim[i] = b->pixdim[i];
    v.integer_levels = b->dtype == U8 || b->dtype == U16;
    return v;
}

static constexpr int SEAM_BUCKETS_MAX = 256;

static dcf_status batch_set_tiles(dcf_ctx *ctx, dcf_batch *b, int tw, int th, int ctas, int chunk)
{
    if (tw < 1 || th < 1 || tw * th > TILE_MAX_PIX || tile_smem_bytes(tw, th, 1) > 48 * 1024)
        return set_err(ctx, DCF_ERR_INVALID, "tile %dx%d (at most %d pixels, 48 KiB of shared memory)", tw, th,
                       TILE_MAX_PIX);
    const int maxc = batch_max_ctas_per_sm(b->dtype, tw, th);
    if (maxc < 1) return set_err(ctx, DCF_ERR_INVALID, "tile %dx%d does not fit on an SM", tw, th);
    if (ctas < 1 || ctas > maxc) ctas = maxc;
    if (chunk < 1) chunk = 1;
    std::vector<BatchTile> tl;
    for (int i = 0; i < b->count; i++)
        for (int y = 0; y < b->imgs[i].H; y += th)
            for (int x = 0; x < b->imgs[i].W; x += tw) tl.push_back(BatchTile{i, x, y});
    if (tl.size() > b->tiles_cap) {
        if (b->d_tiles) CU(cudaFree(b->d_tiles));
        b->d_tiles = nullptr;
        b->tiles_cap = 0;
        CU(dmalloc(ctx, &b->d_tiles, tl.size() * sizeof(BatchTile)));
        b->tiles_cap = tl.size();
    }
    CU(cudaMemcpyAsync(b->d_tiles, tl.data(), tl.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    {
        Geom tg{};
        tg.conn = b->conn;
        tg.tw = tw;
        tg.th = th;
        const long long cap = batch_seam_edge_bound(tg, b->imgs.data(), b->count);
        const size_t need = seam_edges_bytes(cap, SEAM_BUCKETS_MAX);
        if (need > b->seam_bytes) {
            batch_drop_graph(b);
            if (b->seam_mem) CU(cudaFree(b->seam_mem));
            b->seam_mem = nullptr;
            b->seam_bytes = 0;
            CU(dmalloc(ctx, &b->seam_mem, need));
            b->seam_bytes = need;
        }
        // laid out for the largest bucket count, so set_merge can change it in place
        b->seam = seam_edges_carve(b->seam_mem, cap, SEAM_BUCKETS_MAX);
        b->seam.buckets = b->seam_buckets;
    }
    b->ntiles = (int)tl.size();
    b->tw = tw;
    b->th = th;
    b->ctas = ctas;
    b->chunk = chunk;
    batch_drop_graph(b);
    return DCF_OK;
}

static dcf_status batch_ensure_rest(dcf_ctx *ctx, dcf_batch *b, unsigned R)
{
    const size_t need = attr_rest_bytes(b->group, R);
    if (need <= b->rest_bytes) return DCF_OK;
    batch_drop_graph(b);
    CU(cudaStreamSynchronize(ctx->stream));
    if (b->rest_mem) CU(cudaFree(b->rest_mem));
    b->rest_mem = nullptr;
    b->rest_bytes = 0;
    CU(dmalloc(ctx, &b->rest_mem, need));
    b->rest_bytes = need;
    return DCF_OK;
}

// Enqueue the build + attributes (+ filter, + spectra) of every cutout.  graph:
// the pointer-jumping phase uses the fixed capacity; otherwise the rest count is
// read back (a host synchronisation) and the scratch sized from it.
static dcf_status batch_forward(dcf_ctx *ctx, dcf_batch *b, const void *px, float *filtered, double *spectra,
                                bool graph)
{
    cudaStream_t s = ctx->stream;
    const int sm = ctx->sm_count;
    const TreeView v = batch_view(b);
    CU(cudaMemsetAsync(b->d_misc + 2, 0xFF, sizeof(unsigned), s));
    CU(cudaMemsetAsync(b->d_misc + 3, 0, 2 * sizeof(unsigned), s));
    CU(cudaMemsetAsync(b->d_nodes, 0, sizeof(unsigned long long), s));
    launch_stats(b->dtype, px, b->N, b->d_misc + 2, b->d_misc + 3, b->d_misc + 4, sm, s);
    launch_batch_build(b->dtype, px, v.g, b->d_imgs, b->d_tiles, b->ntiles, b->chunk, b->d_misc, b->gval, b->node,
                       b->parent, b->isroot, b->d_nodes, b->nodes, ctx->d_err, b->ctas, b->seam, sm, s);
    CU(attr_zero(b->attr, b->nodes, b->d_nodes, (size_t)b->N, sm, s));
    launch_batch_attr_pixels(v.g, b->d_imgs, b->d_tiles, b->ntiles, b->gval, b->parent, b->isroot, b->attr, sm, s);
    unsigned *count = b->d_misc + 1;
    launch_attributes_up(v, b->attr, count, b->up_steps, ctx->d_err, sm, s);
    if (graph) {
        launch_attributes_rest_cap(v, b->attr, b->rest_cap, count, b->rest_mem, ctx->d_err, sm, s);
    } else {
        dcf_status st = check_launch(ctx, 12);
        if (st != DCF_OK) return st;
        unsigned R = 0;
        CU(cudaMemcpyAsync(&R, count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
        if (R > 0) {
            if ((st = batch_ensure_rest(ctx, b, R)) != DCF_OK) return st;
            launch_attributes_rest(v, b->attr, R, count, b->rest_mem, ctx->d_err, sm, s);
        }
        // capacity of later graph runs: twice what this input needed
        unsigned cap = R < (1u << 15) ? (1u << 16) : 2 * R;
        if (cap > b->rest_cap) b->rest_cap = cap;
    }
    const dcf_op_set &o = b->ops;
    if (o.filter_attr >= 0) {
        FilterWork w{};
        w.flag = b->flag;
        w.target = b->target;
        if (filtered)
            launch_filter(v, b->attr, o.filter_attr, DCF_RULE_DIRECT, o.lambda, false, filtered, w, b->N, ctx->d_err,
                          sm, s);
        else
            launch_direct_targets(v, b->attr, o.filter_attr, o.lambda, w, ctx->d_err, sm, s);
    }
    if (o.spec_attr1 >= 0 && spectra) {
        CU(cudaMemsetAsync(spectra, 0, (size_t)b->count * o.n1 * o.n2 * 8, s));
        launch_batch_spectrum(v.g, b->d_imgs, b->d_tiles, b->ntiles, b->parent, b->isroot, b->gval, b->attr,
                              o.spec_attr1, b->lvec, o.n1, o.spec_attr2 == 0 ? -1 : o.spec_attr2, b->lvec + o.n1,
                              o.n2, b->pixdim, spectra, sm, s);
    }
    return check_launch(ctx, 6);
}

// device error bits and NaN count after a run; *capacity: the graph's
// pointer-jumping list overflowed
static dcf_status batch_check(dcf_ctx *ctx, dcf_batch *b, bool *capacity)
{
    CU(cudaStreamSynchronize(ctx->stream));
    unsigned err = 0, misc[5];
    CU(cudaMemcpy(&err, ctx->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(misc, b->d_misc, sizeof(misc), cudaMemcpyDeviceToHost));
    if (capacity) *capacity = (err & DEVERR_CAPACITY) != 0;
    if (err) CU(cudaMemset(ctx->d_err, 0, sizeof(unsigned)));
    if (capacity && *capacity) {
        // the truncated list also trips the pointer-jumping link check; the run is
        // redone without the graph, which reports any genuine error
        err = 0;
        const unsigned R = misc[1];
        b->rest_cap = R > b->rest_cap ? 2 * R : 2 * b->rest_cap;
    }
    if (err) return set_err(ctx, DCF_ERR_TIMEOUT, "device loop bound exceeded (bits 0x%x)", err);
    if (misc[4]) return set_err(ctx, DCF_ERR_NAN, "batch holds %u NaN values", misc[4]);
    return DCF_OK;
}

static int spec_rule_error(dcf_ctx *ctx, int group, int a1, int a2, int n1, int n2, const float *l1, const float *l2)
{
    if (a1 < 0) return DCF_OK;
    if (a1 >= DCF_NUM_ATTRIBUTES || (a1 != 0 && ATTR_GROUP[a1] != group))
        return set_err(ctx, DCF_ERR_INVALID, "spectrum attribute %d is not in the batch's group", a1);
    if (a1 == 0 && a2 != 0) return set_err(ctx, DCF_ERR_INVALID, "the attribute with the highest index must come first");
    if (a2 != 0 && (a2 < 0 || a2 >= DCF_NUM_ATTRIBUTES || ATTR_GROUP[a2] != group))
        return set_err(ctx, DCF_ERR_INVALID, "both 2-D spectrum attributes must be in one group");
    if (n1 < 1 || n2 < 1 || !l1 || !l2) return set_err(ctx, DCF_ERR_INVALID, "bad lambda vectors");
    return DCF_OK;
}

extern "C" {

dcf_status dcf_batch_create(dcf_ctx *ctx, int count, const uint32_t *widths, const uint32_t *heights, int dtype,
                            int connectivity, int attr_idx, const float *pixdim, dcf_batch **out)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !out || !widths || !heights) return DCF_ERR_INVALID;
    *out = nullptr;
    if (count < 1) return set_err(ctx, DCF_ERR_INVALID, "empty batch");
    if (dtype < DCF_U8 || dtype > DCF_F32) return set_err(ctx, DCF_ERR_INVALID, "bad dtype %d", dtype);
    if (connectivity != 4 && connectivity != 8)
        return set_err(ctx, DCF_ERR_INVALID, "batch connectivity must be 4 or 8 (got %d)", connectivity);
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES) return set_err(ctx, DCF_ERR_INVALID, "bad attribute %d", attr_idx);
    dcf_batch *b = new (std::nothrow) dcf_batch();
    if (!b) return DCF_ERR_NOMEM;
    b->ctx = ctx;
    b->merge_bound = ctx->merge_bound;
    b->count = count;
    b->dtype = dtype;
    b->conn = connectivity;
    b->attr_idx = attr_idx;
    b->group = ATTR_GROUP[attr_idx];
    b->up_steps = ctx->up_steps;
    if (pixdim)
        for (int i = 0; i < 3; i++) b->pixdim[i] = pixdim[i];
    std::vector<long long> offs(count);
    long long N = 0;
    b->imgs.resize(count);
    for (int i = 0; i < count; i++) {
        if (widths[i] < 1 || heights[i] < 1 || widths[i] > 0x7FFFFFFF || heights[i] > 0x7FFFFFFF) {
            delete b;
            return set_err(ctx, DCF_ERR_INVALID, "cutout %d is empty or too large", i);
        }
        offs[i] = N;
        b->imgs[i] = BatchImg{N, (int)widths[i], (int)heights[i]};
        N += (long long)widths[i] * heights[i];
        if (N >= 0x7FFFFFFFLL) {
            delete b;
            return set_err(ctx, DCF_ERR_INVALID, "batch too large (limit 2^31-1 pixels)");
        }
    }
    b->N = N;
    static const size_t esize[4] = {1, 2, 4, 4};
    dcf_status st = DCF_OK;
#define BTRY(call)                                                                                            \
    do {                                                                                                      \
        cudaError_t _e = (call);                                                                              \
        if (_e != cudaSuccess) {                                                                              \
            st = set_err(ctx, _e == cudaErrorMemoryAllocation ? DCF_ERR_NOMEM : DCF_ERR_CUDA, "%s: %s", #call, \
                         cudaGetErrorString(_e));                                                             \
            goto fail;                                                                                        \
        }                                                                                                     \
    } while (0)
    BTRY(dmalloc(ctx, &b->d_imgs, count * sizeof(BatchImg)));
    BTRY(dmalloc(ctx, &b->d_offs, count * sizeof(long long)));
    BTRY(dmalloc(ctx, &b->d_misc, 8 * sizeof(unsigned) + sizeof(unsigned long long)));
    b->d_nodes = (unsigned long long *)(b->d_misc + 8);
    BTRY(dmalloc(ctx, &b->pixels, (size_t)N * esize[dtype]));
    BTRY(dmalloc(ctx, &b->gval, (size_t)N * 4));
    BTRY(dmalloc(ctx, &b->node, (size_t)N * 8));
    BTRY(dmalloc(ctx, &b->parent, (size_t)N * 4));
    BTRY(dmalloc(ctx, &b->isroot, (size_t)N));
    BTRY(dmalloc(ctx, &b->nodes, node_list_bytes(N)));
    BTRY(dmalloc(ctx, &b->attr_mem, attr_bytes(b->group, (size_t)N)));
    attr_carve(b->attr, b->group, dtype == U8 || dtype == U16, false, (size_t)N, b->attr_mem);
    BTRY(cudaMemcpy(b->d_imgs, b->imgs.data(), count * sizeof(BatchImg), cudaMemcpyHostToDevice));
    BTRY(cudaMemcpy(b->d_offs, offs.data(), count * sizeof(long long), cudaMemcpyHostToDevice));
    BTRY(cudaMemset(b->d_misc, 0, 8 * sizeof(unsigned) + sizeof(unsigned long long)));
    if ((st = batch_set_tiles(ctx, b, 64, 64, 0, 1)) != DCF_OK) goto fail;
    *out = b;
    return DCF_OK;
fail:
    dcf_batch_destroy(b);
    return st;
#undef BTRY
}

dcf_status dcf_batch_destroy(dcf_batch *b)
{
    if (!b) return DCF_ERR_INVALID;
    if (b->ctx) cudaStreamSynchronize(b->ctx->stream);
    batch_drop_graph(b);
    void *bufs[] = {b->d_imgs, b->d_offs, b->d_tiles, b->d_misc, b->pixels, b->gval, b->node, b->parent, b->isroot,
                    b->nodes, b->attr_mem, b->rest_mem, b->flag, b->target, b->filtered, b->spectra, b->lvec, b->adj_acc,
                    b->adj_io, b->adj_w, b->seam_mem};
    for (void *p : bufs)
        if (p) cudaFree(p);
    delete b;
    return DCF_OK;
}

dcf_status dcf_batch_info(const dcf_batch *b, uint64_t *total_pixels, uint64_t *num_nodes, int *schedule,
                          uint64_t *graph_kernels)
{
    if (!b) return DCF_ERR_INVALID;
    if (total_pixels) *total_pixels = (uint64_t)b->N;
    if (num_nodes) {
        unsigned long long n = 0;
        if (b->valid) {
            cudaStreamSynchronize(b->ctx->stream);
            cudaMemcpy(&n, b->d_nodes, sizeof(n), cudaMemcpyDeviceToHost);
        }
        *num_nodes = n;
    }
    if (schedule) {
        schedule[0] = b->tw;
        schedule[1] = b->th;
        schedule[2] = b->ctas;
        schedule[3] = b->chunk;
        schedule[4] = b->seam_buckets;
        schedule[5] = b->up_steps;
    }
    if (graph_kernels) *graph_kernels = b->graph_kernels;
    return DCF_OK;
}

dcf_status dcf_batch_set_schedule(dcf_ctx *ctx, dcf_batch *b, int tile_w, int tile_h, int ctas_per_sm, int chunk)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b) return DCF_ERR_INVALID;
    return batch_set_tiles(ctx, b, tile_w, tile_h, ctas_per_sm, chunk);
}

dcf_status dcf_batch_set_merge(dcf_ctx *ctx, dcf_batch *b, int seam_buckets, int up_steps)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b) return DCF_ERR_INVALID;
    if (seam_buckets < 0 || seam_buckets > SEAM_BUCKETS_MAX)
        return set_err(ctx, DCF_ERR_INVALID, "seam buckets %d (0..%d)", seam_buckets, SEAM_BUCKETS_MAX);
    if (up_steps < 0 || up_steps >= (1 << 24)) return set_err(ctx, DCF_ERR_INVALID, "up_steps %d", up_steps);
    batch_drop_graph(b);
    b->seam_buckets = seam_buckets;
    b->seam.buckets = seam_buckets;
    b->up_steps = up_steps;
    b->rest_cap = 0;  // the pointer-jumping capacity is learned again
    b->valid = false;
    return DCF_OK;
}

dcf_status dcf_batch_autotune(dcf_ctx *ctx, dcf_batch *b, const void *pixels, int on_device, int repeats,
                              double *best_ms)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b || !pixels) return DCF_ERR_INVALID;
    if (repeats < 1) repeats = 1;
    static const size_t esize[4] = {1, 2, 4, 4};
    const void *px = pixels;
    if (!on_device) {
        CU(cudaMemcpyAsync(b->pixels, pixels, (size_t)b->N * esize[b->dtype], cudaMemcpyHostToDevice, ctx->stream));
        px = b->pixels;
    }
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    const bool prof = ctx->prof_on;
    ctx->prof_on = false;
    // time the build phase (queue reset, persistent tile kernel, seams, canonical form)
    auto time_build = [&](double *ms) -> dcf_status {
        const TreeView v = batch_view(b);
        std::vector<float> t;
        for (int r = 0; r <= repeats; r++) {  // the first pass warms up
            cudaEventRecord(e0, ctx->stream);
            launch_batch_build(b->dtype, px, v.g, b->d_imgs, b->d_tiles, b->ntiles, b->chunk, b->d_misc, b->gval,
                               b->node, b->parent, b->isroot, b->d_nodes, b->nodes, ctx->d_err, b->ctas, b->seam,
                               ctx->sm_count, ctx->stream);
            cudaEventRecord(e1, ctx->stream);
            dcf_status st = check_launch(ctx, 4);
            if (st != DCF_OK) return st;
            CU(cudaEventSynchronize(e1));
            float x = 0.f;
            cudaEventElapsedTime(&x, e0, e1);
            if (r) t.push_back(x);
        }
        std::sort(t.begin(), t.end());
        *ms = t[t.size() / 2];
        return DCF_OK;
    };
    struct Cand {
        int tw, th, ctas, chunk;
    };
    static const int shapes[][2] = {{64, 64}, {128, 32}, {64, 32}, {32, 32}};
    Cand best{64, 64, 0, 1};
    double best_t = 1e30;
    dcf_status st = DCF_OK;
    // 1) tile shape at full occupancy, 2) CTAs per SM and queue chunk for that shape
    for (auto &sh : shapes) {
        double ms;
        if ((st = batch_set_tiles(ctx, b, sh[0], sh[1], 0, 1)) != DCF_OK) break;
        if ((st = time_build(&ms)) != DCF_OK) break;
        if (ms < best_t) {
            best_t = ms;
            best = Cand{sh[0], sh[1], b->ctas, 1};
        }
    }
    if (st == DCF_OK) {
        const int maxc = batch_max_ctas_per_sm(b->dtype, best.tw, best.th);
        for (int c : {1, 2, maxc})
            for (int ch : {1, 4}) {
                if (c > maxc || (c == best.ctas && ch == 1)) continue;
                double ms;
                if ((st = batch_set_tiles(ctx, b, best.tw, best.th, c, ch)) != DCF_OK) break;
                if ((st = time_build(&ms)) != DCF_OK) break;
                if (ms < best_t) {
                    best_t = ms;
                    best = Cand{best.tw, best.th, c, ch};
                }
            }
    }
    // 3) seam buckets on the build, 4) bottom-up steps on build + attributes
    int best_buckets = b->seam_buckets, best_up = b->up_steps;
    if (st == DCF_OK) st = batch_set_tiles(ctx, b, best.tw, best.th, best.ctas, best.chunk);
    if (st == DCF_OK) {
        for (int nb : {0, 16, 64}) {
            if (nb == best_buckets) continue;
            double ms;
            b->seam_buckets = b->seam.buckets = nb;
            if ((st = time_build(&ms)) != DCF_OK) break;
            if (ms < best_t) {
                best_t = ms;
                best_buckets = nb;
            }
        }
        b->seam_buckets = b->seam.buckets = best_buckets;
    }
    double best_fwd = 1e30;
    if (st == DCF_OK) {
        const dcf_op_set keep = b->ops;
        b->ops = dcf_op_set{-1, 0.0, -1, nullptr, 0, 0, nullptr, 0, 0};
        for (int up : {2048, 16384, 131072}) {
            b->up_steps = up;
            std::vector<float> t;
            for (int r = 0; r <= repeats && st == DCF_OK; r++) {
                cudaEventRecord(e0, ctx->stream);
                st = batch_forward(ctx, b, px, nullptr, nullptr, false);
                cudaEventRecord(e1, ctx->stream);
                if (st == DCF_OK) st = batch_check(ctx, b, nullptr);
                float x = 0.f;
                cudaEventElapsedTime(&x, e0, e1);
                if (r) t.push_back(x);
            }
            if (st != DCF_OK) break;
            std::sort(t.begin(), t.end());
            if (t[t.size() / 2] < best_fwd) {
                best_fwd = t[t.size() / 2];
                best_up = up;
            }
        }
        b->up_steps = best_up;
        b->ops = keep;
        b->rest_cap = 0;
    }
    ctx->prof_on = prof;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != DCF_OK) return st;
    b->valid = false;  // the timed runs leave no usable state
    if (best_ms) *best_ms = best_t;
    return batch_check(ctx, b, nullptr);
}

dcf_status dcf_batch_run(dcf_ctx *ctx, dcf_batch *b, const void *pixels, int pixels_on_device, const dcf_op_set *ops,
                         float *filtered, double *spectra, int outputs_on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b || !pixels || !ops) return DCF_ERR_INVALID;
    dcf_op_set o = *ops;
    if (o.filter_attr >= DCF_NUM_ATTRIBUTES || (o.filter_attr > 0 && ATTR_GROUP[o.filter_attr] != b->group))
        return set_err(ctx, DCF_ERR_INVALID, "filter attribute %d is not in the batch's group", o.filter_attr);
    if (o.filter_attr < 0) o.filter_attr = -1;
    if (o.spec_attr1 < 0) {
        o.spec_attr1 = -1;
        o.n1 = o.n2 = 0;
    }
    dcf_status st = (dcf_status)spec_rule_error(ctx, b->group, o.spec_attr1, o.spec_attr2, o.n1, o.n2, o.lvec1, o.lvec2);
    if (st != DCF_OK) return st;
    static const size_t esize[4] = {1, 2, 4, 4};
    const size_t N = (size_t)b->N;
    cudaStream_t s = ctx->stream;
    // buffers the requested operations need (allocated once)
    if (o.filter_attr >= 0 && !b->flag) {
        CU(dmalloc(ctx, &b->flag, N));
        CU(dmalloc(ctx, &b->target, N * 4));
    }
    if (filtered && !outputs_on_device && !b->filtered) CU(dmalloc(ctx, &b->filtered, N * 4));
    const size_t nspec = o.spec_attr1 >= 0 ? (size_t)b->count * o.n1 * o.n2 : 0;
    if (spectra && nspec && !outputs_on_device && nspec > b->spectra_cap) {
        batch_drop_graph(b);
        if (b->spectra) CU(cudaFree(b->spectra));
        b->spectra = nullptr;
        b->spectra_cap = 0;
        CU(dmalloc(ctx, &b->spectra, nspec * 8));
        b->spectra_cap = nspec;
    }
    if (o.spec_attr1 >= 0) {
        if ((size_t)(o.n1 + o.n2) > b->lvec_cap) {
            batch_drop_graph(b);
            if (b->lvec) CU(cudaFree(b->lvec));
            b->lvec = nullptr;
            b->lvec_cap = 0;
            CU(dmalloc(ctx, &b->lvec, (size_t)(o.n1 + o.n2) * 4));
            b->lvec_cap = o.n1 + o.n2;
        }
        CU(cudaMemcpyAsync(b->lvec, o.lvec1, (size_t)o.n1 * 4, cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(b->lvec + o.n1, o.lvec2, (size_t)o.n2 * 4, cudaMemcpyHostToDevice, s));
    }
    const void *px = pixels;
    if (!pixels_on_device) {
        CU(cudaMemcpyAsync(b->pixels, pixels, N * esize[b->dtype], cudaMemcpyHostToDevice, s));
        px = b->pixels;
    }
    float *d_filt = filtered ? (outputs_on_device ? filtered : b->filtered) : nullptr;
    double *d_spec = (spectra && nspec) ? (outputs_on_device ? spectra : b->spectra) : nullptr;
    b->ops = o;
    b->valid = false;
    bool capacity = false;
    if (o.use_graph && b->rest_cap > 0) {
        if ((st = batch_ensure_rest(ctx, b, b->rest_cap)) != DCF_OK) return st;
        BatchKey k;
        k.pixels = px;
        k.filtered = d_filt;
        k.spectra = d_spec;
        k.filter_attr = o.filter_attr;
        k.lambda = o.lambda;
        k.a1 = o.spec_attr1;
        k.a2 = o.spec_attr2;
        k.n1 = o.n1;
        k.n2 = o.n2;
        k.tw = b->tw;
        k.th = b->th;
        k.ctas = b->ctas;
        k.chunk = b->chunk;
        k.cap = b->rest_cap;
        k.rest_mem = b->rest_mem;
        dcf_batch::Graph *gr = nullptr;
        for (auto &g : b->graphs)
            if (g.key == k) gr = &g;
        if (!gr) {
            if (b->graphs.size() >= dcf_batch::MAX_GRAPHS) {
                auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                            [](const dcf_batch::Graph &x, const dcf_batch::Graph &y) { return x.used < y.used; });
                cudaGraphExecDestroy(lru->exec);
                cudaGraphDestroy(lru->graph);
                b->graphs.erase(lru);
            }
            const bool prof = ctx->prof_on;
            ctx->prof_on = false;  // no timing events inside the recorded graph
            const uint64_t launches0 = ctx->launches;
            CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            dcf_status fst = batch_forward(ctx, b, px, d_filt, d_spec, true);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            ctx->prof_on = prof;
            ctx->launches = launches0;
            if (fst != DCF_OK) {
                if (g) cudaGraphDestroy(g);
                return fst;
            }
            if (ce != cudaSuccess) return set_err(ctx, DCF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
            dcf_batch::Graph ng;
            ng.key = k;
            ng.graph = g;
            cudaError_t ie = cudaGraphInstantiate(&ng.exec, g, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(g);
                return set_err(ctx, DCF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
            }
            size_t nn = 0;
            CU(cudaGraphGetNodes(g, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            CU(cudaGraphGetNodes(g, nodes.data(), &nn));
            for (auto nd : nodes) {
                cudaGraphNodeType ty;
                if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ng.kernels++;
            }
            b->graphs.push_back(ng);
            gr = &b->graphs.back();
        }
        gr->used = ++b->uses;
        prof_begin(P_BATCH, s);
        CU(cudaGraphLaunch(gr->exec, s));
        prof_end(P_BATCH, s);
        b->graph_kernels = gr->kernels;
        ctx->launches += gr->kernels;
        st = batch_check(ctx, b, &capacity);
        if (st != DCF_OK) return st;
    }
    if (!o.use_graph || b->rest_cap == 0 || capacity) {
        prof_begin(P_BATCH, s);
        st = batch_forward(ctx, b, px, d_filt, d_spec, false);
        prof_end(P_BATCH, s);
        if (st != DCF_OK) return st;
        st = batch_check(ctx, b, nullptr);
        if (st != DCF_OK) return st;
    }
    b->valid = true;
    if (!outputs_on_device) {
        if (filtered) CU(cudaMemcpyAsync(filtered, d_filt, N * 4, cudaMemcpyDeviceToHost, s));
        if (d_spec) CU(cudaMemcpyAsync(spectra, d_spec, nspec * 8, cudaMemcpyDeviceToHost, s));
        CU(cudaStreamSynchronize(s));
    }
    return DCF_OK;
}

__global__ void k_batch_local_parent(long long n, const int *__restrict__ parent, const long long *__restrict__ offs,
                                     int count, long long *out)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (offs[mid] <= p) lo = mid;
            else hi = mid - 1;
        }
        const int q = parent[p];
        out[p] = q < 0 ? -1 : q - offs[lo];
    }
}

dcf_status dcf_batch_parent(dcf_ctx *ctx, dcf_batch *b, int64_t *parent, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b || !parent) return DCF_ERR_INVALID;
    if (!b->valid) return set_err(ctx, DCF_ERR_STATE, "the batch has not been run");
    const size_t N = (size_t)b->N;
    long long *dst = (long long *)parent;
    void *sbuf = nullptr;
    dcf_status st;
    if (!on_device) {
        if ((st = scratch(ctx, 10, N * 8, &sbuf)) != DCF_OK) return st;
        dst = (long long *)sbuf;
    }
    k_batch_local_parent<<<grid_for(b->N, 256, ctx->sm_count), 256, 0, ctx->stream>>>(b->N, b->parent, b->d_offs,
                                                                                      b->count, dst); note_launch();
    if ((st = check_launch(ctx, 1)) != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(parent, dst, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

dcf_status dcf_batch_node_attribute(dcf_ctx *ctx, dcf_batch *b, int attr_idx, double *out, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b || !out) return DCF_ERR_INVALID;
    if (!b->valid) return set_err(ctx, DCF_ERR_STATE, "the batch has not been run");
    if (attr_idx < 0 || attr_idx >= DCF_NUM_ATTRIBUTES || (attr_idx != 0 && ATTR_GROUP[attr_idx] != b->group))
        return set_err(ctx, DCF_ERR_INVALID, "attribute %d is not in the batch's group", attr_idx);
    const size_t N = (size_t)b->N;
    double *dst = out;
    dcf_status st;
    if (!on_device) {
        void *sbuf;
        if ((st = scratch(ctx, 10, N * 8, &sbuf)) != DCF_OK) return st;
        dst = (double *)sbuf;
    }
    launch_node_attr(batch_view(b), b->attr, attr_idx, false, dst, ctx->sm_count, ctx->stream);
    if ((st = check_launch(ctx, 1)) != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(out, dst, N * 8, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

dcf_status dcf_batch_adjoint(dcf_ctx *ctx, dcf_batch *b, const float *grad_filtered, const double *grad_spectra,
                             float *grad_pixels, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !b || !grad_pixels) return DCF_ERR_INVALID;
    if (!b->valid) return set_err(ctx, DCF_ERR_STATE, "the batch has not been run");
    if (b->dtype != F32) return set_err(ctx, DCF_ERR_UNSUPPORTED, "the adjoint needs float32 pixels");
    const dcf_op_set &o = b->ops;
    if (grad_filtered && o.filter_attr < 0) return set_err(ctx, DCF_ERR_STATE, "the last run had no filter");
    if (grad_spectra && o.spec_attr1 < 0) return set_err(ctx, DCF_ERR_STATE, "the last run had no spectrum");
    const size_t N = (size_t)b->N;
    const size_t nspec = (size_t)b->count * o.n1 * o.n2;
    cudaStream_t s = ctx->stream;
    if (!b->adj_acc) CU(dmalloc(ctx, &b->adj_acc, N * 8));
    const float *v = grad_filtered;
    const double *w = grad_spectra;
    float *grad = grad_pixels;
    if (!on_device) {
        if (!b->adj_io) CU(dmalloc(ctx, &b->adj_io, N * 8));
        if (grad_filtered) {
            CU(cudaMemcpyAsync(b->adj_io, grad_filtered, N * 4, cudaMemcpyHostToDevice, s));
            v = b->adj_io;
        }
        if (grad_spectra) {
            if (nspec > b->adj_w_cap) {
                if (b->adj_w) CU(cudaFree(b->adj_w));
                b->adj_w = nullptr;
                b->adj_w_cap = 0;
                CU(dmalloc(ctx, &b->adj_w, nspec * 8));
                b->adj_w_cap = nspec;
            }
            CU(cudaMemcpyAsync(b->adj_w, grad_spectra, nspec * 8, cudaMemcpyHostToDevice, s));
            w = b->adj_w;
        }
        grad = b->adj_io + N;
    }
    CU(cudaMemsetAsync(b->adj_acc, 0, N * 8, s));
    AdjointArgs j;
    j.target = grad_filtered ? b->target : nullptr;
    j.v = v;
    j.w = grad_spectra ? w : nullptr;
    j.a1 = o.spec_attr1;
    j.n1 = o.n1;
    j.a2 = o.spec_attr2 == 0 ? -1 : o.spec_attr2;
    j.n2 = o.n2;
    j.l1 = b->lvec;
    j.l2 = b->lvec ? b->lvec + o.n1 : nullptr;
    j.offs = b->d_offs;
    j.count = b->count;
    j.acc = b->adj_acc;
    j.grad = grad;
    launch_adjoint(batch_view(b), b->attr, j, ctx->sm_count, s);
    dcf_status st = check_launch(ctx, 2);
    if (st != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(grad_pixels, grad, N * 4, cudaMemcpyDeviceToHost, s));
    return sync_and_check(ctx);
}

dcf_status dcf_tree_adjoint(dcf_ctx *ctx, dcf_tree *t, const dcf_op_set *ops, const float *grad_filtered,
                            const double *grad_spectrum, float *grad_pixels, int on_device)
{
    ActiveScope active_scope_(ctx);
    if (!ctx || !t || !ops || !grad_pixels) return DCF_ERR_INVALID;
    if (t->dtype != F32 || t->tree_min)
        return set_err(ctx, DCF_ERR_UNSUPPORTED, "the adjoint needs a max-tree of float32 pixels");
    const dcf_op_set &o = *ops;
    if (grad_filtered) {
        dcf_status st = check_attr(ctx, t, o.filter_attr);
        if (st != DCF_OK) return st;
    }
    if (grad_spectrum) {
        dcf_status st = check_attr(ctx, t, o.spec_attr1);
        if (st != DCF_OK) return st;
        st = (dcf_status)spec_rule_error(ctx, t->attr.group, o.spec_attr1, o.spec_attr2, o.n1, o.n2, o.lvec1, o.lvec2);
        if (st != DCF_OK) return st;
    }
    const size_t N = (size_t)t->g.N;
    const size_t nspec = grad_spectrum ? (size_t)o.n1 * o.n2 : 0;
    cudaStream_t s = ctx->stream;
    dcf_status st;
    // scratch: 1 flag, 2 target, 10 accumulator, 11 lambda vectors + host-side staging
    void *acc, *io;
    const size_t lbytes = grad_spectrum ? ((size_t)(o.n1 + o.n2) * 4 + 255) / 256 * 256 : 0;
    const size_t io_bytes = lbytes + (on_device ? 0 : nspec * 8 + N * 8);
    if ((st = scratch(ctx, 10, N * 8, &acc)) != DCF_OK) return st;
    if ((st = scratch(ctx, 11, io_bytes + 256, &io)) != DCF_OK) return st;
    float *dl = (float *)io;
    double *dw = (double *)((char *)io + lbytes);
    float *dv = (float *)((char *)io + lbytes + nspec * 8);
    float *dgrad = dv + N;
    AdjointArgs j;
    if (grad_filtered) {
        FilterWork w{};
        void *p;
        if ((st = scratch(ctx, 1, N, &p)) != DCF_OK) return st;
        w.flag = (unsigned char *)p;
        if ((st = scratch(ctx, 2, N * 4, &p)) != DCF_OK) return st;
        w.target = (int *)p;
        launch_direct_targets(view_of(t), t->attr, o.filter_attr, o.lambda, w, ctx->d_err, ctx->sm_count, s);
        j.target = w.target;
        j.v = grad_filtered;
        if (!on_device) {
            CU(cudaMemcpyAsync(dv, grad_filtered, N * 4, cudaMemcpyHostToDevice, s));
            j.v = dv;
        }
    }
    if (grad_spectrum) {
        CU(cudaMemcpyAsync(dl, o.lvec1, (size_t)o.n1 * 4, cudaMemcpyHostToDevice, s));
        CU(cudaMemcpyAsync(dl + o.n1, o.lvec2, (size_t)o.n2 * 4, cudaMemcpyHostToDevice, s));
        j.w = grad_spectrum;
        if (!on_device) {
            CU(cudaMemcpyAsync(dw, grad_spectrum, nspec * 8, cudaMemcpyHostToDevice, s));
            j.w = dw;
        }
        j.a1 = o.spec_attr1;
        j.n1 = o.n1;
        j.a2 = o.spec_attr2 == 0 ? -1 : o.spec_attr2;
        j.n2 = o.n2;
        j.l1 = dl;
        j.l2 = dl + o.n1;
    }
    static const long long zero_off = 0;
    j.offs = &zero_off;  // not read with count == 1
    j.count = 1;
    j.acc = (double *)acc;
    j.grad = on_device ? grad_pixels : dgrad;
    CU(cudaMemsetAsync(acc, 0, N * 8, s));
    launch_adjoint(view_of(t), t->attr, j, ctx->sm_count, s);
    if ((st = check_launch(ctx, 4)) != DCF_OK) return st;
    if (!on_device) CU(cudaMemcpyAsync(grad_pixels, dgrad, N * 4, cudaMemcpyDeviceToHost, s));
    return sync_and_check(ctx);
}

}  // extern "C"
