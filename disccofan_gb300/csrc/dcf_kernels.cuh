// Launch interface between the C-ABI layer (dcf_api.cu) and the kernel units.
#pragma once
#include "dcf_internal.cuh"

namespace dcf {

// Per-kernel timing: launchers bracket each kernel group with prof_begin/prof_end,
// which record CUDA events on the launching stream when the calling context has
// profiling switched on (dcf_ctx_set_profiling); otherwise they do nothing.
enum ProfId : int {
    P_STATS = 0, P_TILE, P_SEAM, P_CANON, P_ATTR_PIX, P_ATTR_UP, P_ATTR_REST, P_FLAG, P_RESOLVE, P_JUMP, P_FILTER_OUT,
    P_CHECK, P_SPECTRUM, P_COPY, P_BATCH, P_ADJOINT, P_COUNT
};
void prof_begin(int id, cudaStream_t s);
void prof_end(int id, cudaStream_t s);

constexpr int TILE_THREADS = 256;
constexpr int TILE_MAX_PIX = 4096;             // largest build tile (16-bit local indices)
constexpr long long MERGE_BOUND_SMEM = 1LL << 22;
constexpr long long MERGE_BOUND_GLOBAL = 1LL << 28;

inline int grid_for(long long n, int block, int sm_count)
{
    long long b = (n + block - 1) / block;
    long long cap = (long long)sm_count * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

struct BuildArgs {
    int dtype;
    bool tree_min;
    const void *img;
    Geom g;
    const unsigned *kmax;            // order key of the maximum level (min-tree inversion)
    float *gval;
    unsigned long long *node;        // N node words (build scratch)
    int *parent;
    unsigned char *isroot;
    unsigned long long *num_nodes;
    unsigned *err;
    int sm_count;
};

void launch_stats(int dtype, const void *img, long long n, unsigned *kmin, unsigned *kmax, unsigned *nans,
                  int sm_count, cudaStream_t s);
void launch_build(const BuildArgs &a, cudaStream_t s);

// ---------------------------------------------------------------------------
// attribute records (structure of arrays over pixels; valid at level roots)
// ---------------------------------------------------------------------------
struct AttrBufs {
    int group = -1;
    bool exact_g = false;            // grey-weighted sums kept as exact integers (u8/u16)
    bool has_z = true;               // 3-D image: z extent is accumulated (2-D: fixed [0,1))
    uint32_t *area = nullptr;
    uint32_t *bmin[3] = {nullptr, nullptr, nullptr};
    uint32_t *bmax[3] = {nullptr, nullptr, nullptr};
    unsigned long long *s1[3] = {nullptr, nullptr, nullptr};   // sum x, y, z
    unsigned long long *s2[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // x2 y2 z2 xy yz xz
    void *gw[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // sum g, g^2, g*x, g*y, g*z (i64 or f64)
    int *pending = nullptr;          // children not yet folded in (bottom-up pass)
};

struct TreeView {
    Geom g;
    bool tree_min;
    const unsigned *kmax;            // device: order key of the input's maximum
    const float *gval;
    const int *parent;
    const unsigned char *isroot;
    float pixdim[3];
    bool integer_levels;             // u8/u16 input: level arithmetic is exact in float
};

// Attribute accumulation in two launches: launch_attributes runs the pixel pass and
// the bounded bottom-up fold and counts the nodes left into *count; the caller
// reads that count R and calls launch_attributes_rest with attr_rest_bytes(group, R)
// bytes of device scratch to finish them by pointer jumping.
size_t attr_rest_bytes(int group, size_t R);
void launch_fill_u32(long long n, uint32_t *dst, uint32_t v, int sm_count, cudaStream_t s);
void launch_attributes(const TreeView &t, AttrBufs &a, unsigned *count, int up_steps, unsigned *err, int sm_count,
                       cudaStream_t s);
void launch_attributes_rest(const TreeView &t, AttrBufs &a, unsigned R, unsigned *count, void *scratch, unsigned *err,
                            int sm_count, cudaStream_t s);

// attribute readout of every level root into a double array (NaN elsewhere)
void launch_node_attr(const TreeView &t, const AttrBufs &a, int attr, bool area, double *out, int sm_count,
                      cudaStream_t s);

// ---------------------------------------------------------------------------
// operations
// ---------------------------------------------------------------------------
struct FilterWork {
    unsigned char *flag = nullptr;  // per pixel: survive bit (valid at level roots)
    int *target = nullptr;          // per pixel: resolved node / topmost removed ancestor
    unsigned *kept = nullptr;       // max rule: node has a surviving descendant-or-self
    int *jump = nullptr, *jump2 = nullptr;   // pointer-jumping double buffers
    int *best2 = nullptr;
    double *acc = nullptr, *acc2 = nullptr;
    unsigned *remaining = nullptr;  // exact subtractive rule: nodes still unresolved
};

void launch_filter(const TreeView &t, const AttrBufs &a, int attr, int rule, double lambda, bool extract,
                   float *out, const FilterWork &w, long long depth_bound, unsigned *err, int sm_count,
                   cudaStream_t s);
void launch_check(const TreeView &t, const AttrBufs &a, int attr, float *out, int sm_count, cudaStream_t s);
void launch_spectrum(const TreeView &t, const AttrBufs &a, int a1, const float *l1, int n1, int a2,
                     const float *l2, int n2, double *spec, int sm_count, cudaStream_t s);
void launch_level_out(const TreeView &t, float *out, int sm_count, cudaStream_t s);

}  // namespace dcf
