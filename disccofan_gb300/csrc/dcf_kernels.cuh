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
// counts one kernel launch for the context whose API call is running on this thread
// (dcf_ctx_launch_count); every launch site calls it right after the launch
void note_launch();

constexpr int TILE_THREADS = 256;        // tile build CTAs with 64-bit shared node words (u32/f32)
constexpr int TILE_THREADS_NARROW = 128; // with 32-bit words (u8/u16): more tiles resident per SM
constexpr int TILE_MAX_PIX = 4096;             // largest build tile (16-bit local indices)
constexpr long long MERGE_BOUND_SMEM = 1LL << 22;
constexpr long long MERGE_BOUND_GLOBAL = 1LL << 28;
__host__ __device__ inline long long merge_bound_smem(const Geom &g)
{
    return g.merge_bound > 0 ? g.merge_bound : MERGE_BOUND_SMEM;
}
__host__ __device__ inline long long merge_bound_global(const Geom &g)
{
    return g.merge_bound > 0 ? g.merge_bound : MERGE_BOUND_GLOBAL;
}

// dynamic shared memory of one tile build (padded node words); word_bytes 8
// (u32/f32 images) or 4 (u8/u16: 16-bit level and parent)
inline size_t tile_smem_bytes(int tw, int th, int td, int word_bytes = 8)
{
    return (size_t)(tw + 1) * th * td * word_bytes;
}
// launch shape of the tile kernels per pixel type: u8/u16 tiles use 32-bit shared
// words and 128-thread CTAs (16.5 KB for 4096 pixels: 12 resident per SM, the
// register file's limit at 40 registers a thread), u32/f32 tiles 64-bit words and
// 256 threads (33 KB; 5 per SM, where they run without register spills)
template <typename T> struct TileCfg {
    static constexpr bool narrow = sizeof(T) <= 2;
    static constexpr int threads = narrow ? TILE_THREADS_NARROW : TILE_THREADS;
    static constexpr int min_blocks = narrow ? 12 : 5;
    static constexpr int word_bytes = narrow ? 4 : 8;
};

// the level roots of a tree (TreeView::nodes, TreeView::num_nodes)
struct NodeSet {
    const int *nodes;
    const unsigned long long *num;
};

// Grid-stride loop over the level roots that launch_canon listed (nodes[0 ..
// *num_nodes), ascending): `u` is the node's pixel index.  `continue` in the body
// moves to the next node.
#define NODE_LOOP(u, nodes, num_nodes)                                                                         \
    for (long long _nl_i = blockIdx.x * (long long)blockDim.x + threadIdx.x, _nl_m = (long long)*(num_nodes); \
         _nl_i < _nl_m; _nl_i += (long long)gridDim.x * blockDim.x)                                           \
        for (int u = (nodes)[_nl_i], _nl_once = 1; _nl_once; _nl_once = 0)

inline int grid_for(long long n, int block, int sm_count)
{
    long long b = (n + block - 1) / block;
    long long cap = (long long)sm_count * 32;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// Seam merge of tile forests.  The cross-tile edges are collected with their level
// min(key p, key q); with buckets > 0 they are merged in ascending level order, in
// `buckets` ranges of about equal size: the lowest edges zip the long root paths
// (trunks) of neighbouring tiles first, so later, higher edges stop where the chains
// are already one instead of each walking the trunk again.  buckets == 0 merges
// every edge at once, one connect per thread.  A collect kernel (one per
// enumeration: whole image or batch) appends the edges and histograms the levels'
// top 16 bits; launch_seam_buckets splits and merges them.
constexpr int SEAM_BINS = 65536;
struct SeamEdges {
    int2 *pq = nullptr;              // collected edges (capacity cap)
    unsigned *lvl = nullptr;
    int2 *sorted = nullptr;          // edges grouped by bucket
    unsigned *hist = nullptr;        // SEAM_BINS counts of level >> 16
    unsigned short *bin_bucket = nullptr;  // SEAM_BINS
    unsigned *bstart = nullptr;      // buckets + 1 (exclusive prefix), then the buckets' fill counters
    unsigned *count = nullptr;
    long long cap = 0;
    int buckets = 0;
};
// layout for up to `buckets` buckets (e.buckets may later be set to any value up to it)
size_t seam_edges_bytes(long long cap, int buckets);
SeamEdges seam_edges_carve(void *mem, long long cap, int buckets);
// bound on the cross-tile edges of a tile grid (outward offsets per face)
long long seam_edge_bound(const Geom &g, long long ntiles);
void launch_seam_buckets(SeamEdges &e, unsigned long long *node, long long n, long long merge_bound, unsigned *err,
                         int sm_count, cudaStream_t s);

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
    int *nodes;                      // level-root list (node_list_bytes(N) bytes)
    unsigned *err;
    int sm_count;
    SeamEdges seam;                  // level-ordered seam merge scratch (buckets == 0: direct merge)
};
// canonical form, then the level roots listed in ascending index order into
// `nodes` (a buffer of node_list_bytes(N) bytes: the list, then chunk counts)
size_t node_list_bytes(long long n);
void launch_canon(unsigned long long *node, const Geom &g, int *parent, unsigned char *isroot,
                  unsigned long long *num_nodes, int *nodes, unsigned *err, int sm_count, cudaStream_t s);

void launch_stats(int dtype, const void *img, long long n, unsigned *kmin, unsigned *kmax, unsigned *nans,
                  int sm_count, cudaStream_t s);
void launch_build(const BuildArgs &a, cudaStream_t s);

// ---------------------------------------------------------------------------
// batches of 2-D cutouts: pixels of all cutouts concatenated, cutout i at element
// off_i; trees use global indices, so the node-parallel passes run unchanged on
// the concatenation
// ---------------------------------------------------------------------------
struct BatchImg {
    long long off;
    int W, H;
};
struct BatchTile {
    int img, x0, y0;
};
// persistent work-queue tile build (grid = sm_count * ctas_per_sm CTAs, `chunk`
// tiles per queue grab), seam merge inside each cutout, canonical form
void launch_batch_build(int dtype, const void *img, const Geom &bg, const BatchImg *imgs, const BatchTile *tiles,
                        int ntiles, int chunk, unsigned *next, float *gval, unsigned long long *node, int *parent,
                        unsigned char *isroot, unsigned long long *num_nodes, int *nodes, unsigned *err,
                        int ctas_per_sm, SeamEdges &seam, int sm_count, cudaStream_t s);
// bound on a batch's cross-tile edges (capacity of its SeamEdges)
long long batch_seam_edge_bound(const Geom &bg, const BatchImg *imgs_host, int count);

// ---------------------------------------------------------------------------
// attribute records (indexed by pixel; valid at level roots)
// ---------------------------------------------------------------------------
// One 32-bit field of the records: element i at p[i * stride].  The 32-bit fields of
// a node are interleaved so that a pass touching one node's record reads one
// 32-byte sector instead of one sector per field: in the extent group the record
// is REC1_WORDS words (area, pending, bmin x/y/z, bmax x/y/z), in the other groups
// area and pending share one 8-byte pair.  The 64-bit moment sums stay one array
// per field.
template <typename T>
struct Field {
    T *p = nullptr;
    int stride = 1;
    __host__ __device__ T &operator[](long long i) const { return p[i * stride]; }
    __host__ __device__ T *operator+(long long i) const { return p + i * stride; }
};
constexpr int REC1_WORDS = 8;  // extent-group record: area, pending, bmin[3], bmax[3]

struct AttrBufs {
    int group = -1;
    bool exact_g = false;            // grey-weighted sums kept as exact integers (u8/u16)
    bool has_z = true;               // 3-D image: z extent is accumulated (2-D: fixed [0,1))
    Field<uint32_t> area;
    Field<uint32_t> bmin[3];
    Field<uint32_t> bmax[3];
    unsigned long long *s1[3] = {nullptr, nullptr, nullptr};   // sum x, y, z
    unsigned long long *s2[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // x2 y2 z2 xy yz xz
    void *gw[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // sum g, g^2, g*x, g*y, g*z (i64 or f64)
    Field<int> pending;              // children not yet folded in (bottom-up pass)
    unsigned char *single = nullptr; // node has exactly one child (bottom-up pass)
    bool grey = true;                // inertia group: accumulate the grey-weighted sums too
};

// the record of every level root in `ns` set to its start value: zero area, pending
// and sums, empty bounding boxes (minimum all-ones), in 2-D the fixed z extent
// [0, 1).  Only level roots' records are ever read or written (pixels add into
// their node's), so the other pixels' records are left as they are; n bounds the
// node count (grid size)
void launch_attr_init(const AttrBufs &a, NodeSet ns, long long n, int sm_count, cudaStream_t s);

// Fields a pass must move: z moments only in 3-D; grey-weighted sums for the wmean
// group, and for the inertia group only when asked (its attributes 13-17 use the
// geometric moments alone; the sums feed the tree file's weighted centroids); the
// sum of squared grey levels is read by no attribute.
__host__ __device__ inline bool s1_used(const AttrBufs &a, int d) { return d < 2 || a.has_z; }
__host__ __device__ inline bool s2_used(const AttrBufs &a, int d) { return d == 0 || d == 1 || d == 3 || a.has_z; }
__host__ __device__ inline bool gw_used(const AttrBufs &a, int d)
{
    return (a.group == 3 || (a.group == 4 && a.grey)) && d != 1 && (d != 4 || a.has_z);
}

struct TreeView {
    Geom g;
    bool tree_min;
    const unsigned *kmax;            // device: order key of the input's maximum
    const float *gval;
    const int *parent;
    const unsigned char *isroot;
    const int *nodes;                // the level roots, ascending (launch_canon)
    const unsigned long long *num_nodes;  // device: their count
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

// the bottom-up part of launch_attributes alone (after a pixel pass done elsewhere)
void launch_attributes_up(const TreeView &t, AttrBufs &a, unsigned *count, int up_steps, unsigned *err, int sm_count,
                          cudaStream_t s);
// launch_attributes_rest without the host read of the count: scratch sized for
// `cap` nodes (attr_rest_bytes(group, cap)); a count above cap raises
// DEVERR_CAPACITY and leaves the records incomplete.  Issues no host
// synchronisation, so it can be captured in a CUDA graph.
void launch_attributes_rest_cap(const TreeView &t, AttrBufs &a, unsigned cap, unsigned *count, void *scratch,
                                unsigned *err, int sm_count, cudaStream_t s);
int batch_max_ctas_per_sm(int dtype, int tw, int th);
// per-pixel contributions of a batch, walked tile by tile (coordinates inside the cutout)
void launch_batch_attr_pixels(const Geom &bg, const BatchImg *imgs, const BatchTile *tiles, int ntiles,
                              const float *gval, const int *parent, const unsigned char *isroot, AttrBufs &a,
                              int sm_count, cudaStream_t s);

// attribute readout of every level root into a double array (NaN elsewhere);
// attr >= INERTIA_COL0 (INERTIA_COL0 + k): the inertia group's tree-file centroid
// column k (inertia_column)
constexpr int INERTIA_COL0 = 100;
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

// out: N pixels of out_dtype (F32; U8 or U16 only for trees of u8 / u16 images)
void launch_filter(const TreeView &t, const AttrBufs &a, int attr, int rule, double lambda, bool extract,
                   void *out, const FilterWork &w, long long depth_bound, unsigned *err, int sm_count,
                   cudaStream_t s, int out_dtype = F32);
void launch_check(const TreeView &t, const AttrBufs &a, int attr, float *out, int sm_count, cudaStream_t s);
void launch_spectrum(const TreeView &t, const AttrBufs &a, int a1, const float *l1, int n1, int a2,
                     const float *l2, int n2, double *spec, int sm_count, cudaStream_t s);
void launch_level_out(const TreeView &t, float *out, int sm_count, cudaStream_t s);
// CSL segmentation (csl.c:27-124) into three per-pixel float images; lv: n lambdas
// (device, with the leading 0); work: csl_work_bytes(N) bytes; synchronises the
// stream between its rounds
size_t csl_work_bytes(long long n);
void launch_csl(const TreeView &t, const AttrBufs &a, int attr, const float *lv, int n, float *contrast, float *scale,
                float *luminance, void *work, unsigned *remaining, int sm_count, cudaStream_t s);
// per-cutout 2-D spectra of a batch, spec[img*n1*n2 + s1 + s2*n1] (accumulated)
void launch_batch_spectrum(const Geom &bg, const BatchImg *imgs, const BatchTile *tiles, int ntiles, const int *parent,
                           const unsigned char *isroot, const float *gval, const AttrBufs &a, int a1, const float *l1,
                           int n1, int a2, const float *l2, int n2, const float *pixdim, double *spec, int sm_count,
                           cudaStream_t s);

// Adjoint of out = direct-rule filter (v = d loss / d out, per pixel; target =
// the resolved surviving node of every level root, from launch_filter) and of
// spec = 2-D pattern spectra (w = d loss / d spec, per cutout), with the tree
// held fixed: d loss / d level(u) is accumulated in acc (double, per pixel,
// zeroed by the caller) at the level root u that carries each node's level, then
// written to grad (float).  `offs` lists the first pixel of each of `count`
// cutouts (count = 1, offs = {0} for one image).
struct AdjointArgs {
    const int *target = nullptr;     // null: no filter term
    const float *v = nullptr;
    const double *w = nullptr;       // null: no spectrum term
    int a1 = 0, n1 = 0, a2 = 0, n2 = 0;
    const float *l1 = nullptr, *l2 = nullptr;
    const long long *offs = nullptr;
    int count = 1;
    double *acc = nullptr;
    float *grad = nullptr;
};
void launch_adjoint(const TreeView &t, const AttrBufs &a, const AdjointArgs &j, int sm_count, cudaStream_t s);
// direct rule up to the resolved targets (flag + resolve), no output pass
void launch_direct_targets(const TreeView &t, const AttrBufs &a, int attr, double lambda, const FilterWork &w,
                           unsigned *err, int sm_count, cudaStream_t s);

}  // namespace dcf
