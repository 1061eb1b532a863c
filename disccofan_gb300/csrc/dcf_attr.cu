// Attribute accumulation and readout (the reference's attribute vtable,
// attributes.c:47-880 + 1201-1248, and its merges during flooding, flood.c:239-240,
// re-designed as two passes over the finished tree):
//
//   k_attr_pixels  every pixel adds its own contribution (area, bounding box,
//                  coordinate and grey-weighted moments) to its node's record;
//                  area updates are warp-aggregated (lanes of one flat zone add once).
//                  Level roots count their children in `pending`.
//   k_mark_leaves  nodes without children are tagged (pending = -1), nodes with
//                  one child flagged (`single`).
//   k_attr_up      bottom-up fold: a thread starts at every leaf, adds its record
//                  into the parent, and only the thread that brings a parent's
//                  pending count to zero continues upward with the completed record.
//
// Coordinate moments are summed as exact 64-bit integers (the reference sums them in
// double, which is exact below 2^53); grey-weighted moments are exact 64-bit integers
// for 8/16-bit images and doubles otherwise.  Readouts (k_node_attr and the device
// function attr_value) follow the reference's expressions operand by operand,
// including which factors are float and which double.
#include <cstdlib>

#include "dcf_kernels.cuh"
#include "dcf_attr_eval.cuh"

namespace dcf {

template <int G, bool EXACT>
__global__ void k_attr_pixels(const float *__restrict__ gval, Geom g, const int *__restrict__ parent,
                              const unsigned char *__restrict__ isroot, AttrBufs a)
{
    // whole warps iterate together (uniform trip count), so the match below always
    // has the full warp: the area of lanes in one flat zone is added once
    const int lane = threadIdx.x & 31;
    const long long wstride = (long long)gridDim.x * blockDim.x;
    for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane; base < g.N; base += wstride) {
        const long long p = base + lane;
        const bool valid = p < g.N;
        const int par = valid ? parent[p] : NONE;
        const bool root = valid && isroot[p];
        const int node = valid ? (root ? (int)p : par) : -2;
        if (root && par != NONE) atomicAdd(a.pending + par, 1);
        unsigned grp = __match_any_sync(0xffffffffu, node);
        if (valid && lane == __ffs(grp) - 1) atomicAdd(a.area + node, (unsigned)__popc(grp));
        if (G == 0 || !valid) continue;
        // coordinates: one division per warp for its first pixel; lanes add their
        // offset unless the warp's 32 pixels run past the end of a row
        const long long zb = base / g.WH, rem = base - zb * g.WH;
        const long long yb = rem / g.W, xb = rem - yb * g.W;
        const bool one_row = xb + 31 < g.W;  // warp-uniform
        unsigned x, y, z;
        if (one_row) {
            x = (unsigned)xb + lane;
            y = (unsigned)yb;
            z = (unsigned)zb;
        } else {
            x = (unsigned)(p % g.W);
            y = (unsigned)((p / g.W) % g.H);
            z = (unsigned)(p / g.WH);
        }
        if (G == 1) {
            // lanes of one node reduce first; their leader issues the atomics.  Within
            // one row the group's x range is its first and last lane.
            unsigned mnx, mxx, mny, mxy, mnz, mxz;
            if (one_row) {
                mnx = (unsigned)xb + (unsigned)(__ffs(grp) - 1);
                mxx = (unsigned)xb + (unsigned)(32 - __clz(grp));
                mny = y;
                mxy = y + 1;
                mnz = z;
                mxz = z + 1;
            } else {
                mnx = __reduce_min_sync(grp, x);
                mny = __reduce_min_sync(grp, y);
                mxx = __reduce_max_sync(grp, x + 1);
                mxy = __reduce_max_sync(grp, y + 1);
                mnz = __reduce_min_sync(grp, z);
                mxz = __reduce_max_sync(grp, z + 1);
            }
            if (lane == __ffs(grp) - 1) {
                atomicMin(a.bmin[0] + node, mnx);
                atomicMin(a.bmin[1] + node, mny);
                atomicMax(a.bmax[0] + node, mxx);
                atomicMax(a.bmax[1] + node, mxy);
                if (a.has_z) {
                    atomicMin(a.bmin[2] + node, mnz);
                    atomicMax(a.bmax[2] + node, mxz);
                }
            }
            continue;
        }
        if (G == 2 || G == 4) {
            atomicAdd(a.s1[0] + node, (unsigned long long)x);
            atomicAdd(a.s1[1] + node, (unsigned long long)y);
            if (a.has_z) atomicAdd(a.s1[2] + node, (unsigned long long)z);
        }
        if (G == 4) {
            atomicAdd(a.s2[0] + node, (unsigned long long)x * x);
            atomicAdd(a.s2[1] + node, (unsigned long long)y * y);
            atomicAdd(a.s2[3] + node, (unsigned long long)x * y);
            if (a.has_z) {
                atomicAdd(a.s2[2] + node, (unsigned long long)z * z);
                atomicAdd(a.s2[4] + node, (unsigned long long)y * z);
                atomicAdd(a.s2[5] + node, (unsigned long long)x * z);
            }
        }
        if (G == 3 || (G == 4 && a.grey)) {
            const float gv = gval[p];
            if (EXACT) {
                long long gi = (long long)gv;
                atomicAdd((unsigned long long *)a.gw[0] + node, (unsigned long long)gi);
                atomicAdd((unsigned long long *)a.gw[2] + node, (unsigned long long)(gi * (long long)x));
                atomicAdd((unsigned long long *)a.gw[3] + node, (unsigned long long)(gi * (long long)y));
                if (a.has_z) atomicAdd((unsigned long long *)a.gw[4] + node, (unsigned long long)(gi * (long long)z));
            } else {
                const double gd = (double)gv;
                atomicAdd((double *)a.gw[0] + node, gd);
                atomicAdd((double *)a.gw[2] + node, gd * (double)x);
                atomicAdd((double *)a.gw[3] + node, gd * (double)y);
                if (a.has_z) atomicAdd((double *)a.gw[4] + node, gd * (double)z);
            }
        }
    }
}

// Pixel pass of the area and extent groups on 2-D images, aggregated per tile.
// A node's own pixels are its flat zone, which lies along its level contour: 32
// pixels of a row belong to ~31 different nodes, so aggregating a warp's lanes
// saves little.  Over a 64 x 64 tile the same node recurs (about 2 pixels per
// node and tile on the 16384^2 u16 field), so each CTA first gathers its tile's
// contributions by node in a shared-memory hash table (linear probing on the node
// index; area count and bounding box per slot, shared-memory atomics), then issues
// one set of global atomics per (tile, node).  Children are still counted into
// `pending` with one global atomic per level root.  A slot search that finds the
// table full (it holds as many slots as the tile has pixels, so it cannot be)
// adds straight to the global records instead.
constexpr int AGG_T = 64;                      // tile side
constexpr int AGG_SLOTS = AGG_T * AGG_T;       // one slot per pixel of the tile
constexpr int AGG_THREADS = 512;

// DCF_TILE_AGG=0 in the environment selects the per-warp pixel pass instead (for
// timing comparisons; both give the same records)
static bool agg_enabled()
{
    static const bool on = [] {
        const char *e = getenv("DCF_TILE_AGG");
        return !e || atoi(e) != 0;
    }();
    return on;
}

template <int G>
__host__ __device__ constexpr size_t agg_smem_bytes()
{
    return (size_t)AGG_SLOTS * 4 * (G == 1 ? 6 : 2);
}

template <int G>
__global__ void __launch_bounds__(AGG_THREADS, G == 1 ? 2 : 4)
k_attr_pixels_tiled(Geom g, const int *__restrict__ parent, const unsigned char *__restrict__ isroot, AttrBufs a,
                    int ntx)
{
    extern __shared__ unsigned agg_smem[];
    int *key = (int *)agg_smem;
    unsigned *sarea = agg_smem + AGG_SLOTS;
    unsigned *smnx = sarea + AGG_SLOTS, *smxx = smnx + AGG_SLOTS, *smny = smxx + AGG_SLOTS, *smxy = smny + AGG_SLOTS;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < AGG_SLOTS; i += AGG_THREADS) {
        key[i] = NONE;
        sarea[i] = 0u;
        if (G == 1) {
            smnx[i] = 0xFFFFFFFFu;
            smny[i] = 0xFFFFFFFFu;
            smxx[i] = 0u;
            smxy[i] = 0u;
        }
    }
    __syncthreads();
    const int x0 = (blockIdx.x % ntx) * AGG_T, y0 = (blockIdx.x / ntx) * AGG_T;
    // 16 warps: two per row of 64 pixels, eight rows per step
    const int x = x0 + (warp & 1) * 32 + lane;
    for (int r = warp >> 1; r < AGG_T; r += AGG_THREADS / 64) {
        const int y = y0 + r;
        const bool valid = x < g.W && y < g.H;  // warp-uniform rows; x may end mid-warp
        const long long p = (long long)y * g.W + x;
        const int par = valid ? parent[p] : NONE;
        const bool root = valid && isroot[p];
        const int node = valid ? (root ? (int)p : par) : -2;
        if (root && par != NONE) atomicAdd(a.pending + par, 1);
        const unsigned grp = __match_any_sync(0xffffffffu, node);
        if (!valid || lane != __ffs(grp) - 1) continue;
        const unsigned cnt = __popc(grp);
        const unsigned mnx = (unsigned)x, mxx = (unsigned)(x - lane) + (unsigned)(32 - __clz(grp));
        // slot of `node` (Fibonacci hashing of the index, linear probing)
        unsigned h = ((unsigned)node * 2654435761u) >> 20;
        int slot = NONE;
        for (int probe = 0; probe < AGG_SLOTS; probe++) {
            int k = ((volatile int *)key)[h];
            if (k == NONE) k = atomicCAS(key + h, NONE, node);
            if (k == NONE || k == node) {
                slot = (int)h;
                break;
            }
            h = (h + 1) & (AGG_SLOTS - 1);
        }
        if (slot == NONE) {  // unreachable with one slot per pixel; kept exact regardless
            atomicAdd(a.area + node, cnt);
            if (G == 1) {
                atomicMin(a.bmin[0] + node, mnx);
                atomicMax(a.bmax[0] + node, mxx);
                atomicMin(a.bmin[1] + node, (unsigned)y);
                atomicMax(a.bmax[1] + node, (unsigned)y + 1u);
            }
            continue;
        }
        atomicAdd(sarea + slot, cnt);
        if (G == 1) {
            atomicMin(smnx + slot, mnx);
            atomicMax(smxx + slot, mxx);
            atomicMin(smny + slot, (unsigned)y);
            atomicMax(smxy + slot, (unsigned)y + 1u);
        }
    }
    __syncthreads();
    for (int i = tid; i < AGG_SLOTS; i += AGG_THREADS) {
        const int node = key[i];
        if (node == NONE) continue;
        atomicAdd(a.area + node, sarea[i]);
        if (G == 1) {
            atomicMin(a.bmin[0] + node, smnx[i]);
            atomicMax(a.bmax[0] + node, smxx[i]);
            atomicMin(a.bmin[1] + node, smny[i]);
            atomicMax(a.bmax[1] + node, smxy[i]);
        }
    }
}

// 2-D images: every pixel has z = 0, so the z extent of every node is [0, 1)
__global__ void k_fill_u32(long long n, uint32_t *dst, uint32_t v)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = v;
}

void launch_fill_u32(long long n, uint32_t *dst, uint32_t v, int sm, cudaStream_t s)
{
    k_fill_u32<<<grid_for(n, 256, sm), 256, 0, s>>>(n, dst, v); note_launch();
}

// Start values of the level roots' records.  The extent group's interleaved record
// is two 16-byte stores: area and pending 0, bounding-box minima all-ones, maxima 0;
// in 2-D every pixel has z = 0, so the z extent is the fixed [0, 1).  The other
// groups' area/pending pair is one 8-byte store, then their 64-bit sums.
__global__ void k_attr_init(NodeSet ns, AttrBufs a)
{
    const uint4 lo = make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
    const uint4 hi = a.has_z ? make_uint4(0xFFFFFFFFu, 0u, 0u, 0u) : make_uint4(0u, 0u, 0u, 1u);
    NODE_LOOP(u, ns.nodes, ns.num)
    {
        if (a.group == 1) {
            uint4 *rec = (uint4 *)(a.area.p + (size_t)REC1_WORDS * u);
            rec[0] = lo;
            rec[1] = hi;
            continue;
        }
        *(uint2 *)(a.area.p + 2 * (size_t)u) = make_uint2(0u, 0u);
        for (int d = 0; d < 3; d++)
            if (a.s1[d]) a.s1[d][u] = 0ull;
        for (int d = 0; d < 6; d++)
            if (a.s2[d]) a.s2[d][u] = 0ull;
        for (int d = 0; d < 5; d++)
            if (a.gw[d]) ((unsigned long long *)a.gw[d])[u] = 0ull;
    }
}

void launch_attr_init(const AttrBufs &a, NodeSet ns, long long n, int sm, cudaStream_t s)
{
    k_attr_init<<<grid_for(n, 256, sm), 256, 0, s>>>(ns, a); note_launch();
}

// leaves get pending = -1; nodes with exactly one child are flagged in `single`
__global__ void k_mark_leaves(const int *__restrict__ nodes, const unsigned long long *num_nodes, Field<int> pending,
                              unsigned char *single)
{
    NODE_LOOP(p, nodes, num_nodes)
    {
        const int c = pending[p];
        if (c == 0) pending[p] = -1;
        single[p] = c == 1;
    }
}

// One node's record in registers (the fields the group uses).
template <int G, bool EXACT>
struct Rec {
    uint32_t area;
    uint32_t bmin[3], bmax[3];
    unsigned long long s1[3], s2[6], gw[5];  // gw: integer sums, or the bits of doubles
};

template <int G, bool EXACT>
__device__ __forceinline__ void rec_load(const AttrBufs &a, int u, Rec<G, EXACT> &r)
{
    if (G == 1) {  // the whole interleaved record (REC1_WORDS words) in two 16-byte loads
        const uint4 *rp = (const uint4 *)(a.area + u);
        const uint4 r0 = __ldcg(rp), r1 = __ldcg(rp + 1);
        r.area = r0.x;
        r.bmin[0] = r0.z;
        r.bmin[1] = r0.w;
        r.bmin[2] = r1.x;
        r.bmax[0] = r1.y;
        r.bmax[1] = r1.z;
        r.bmax[2] = r1.w;
        return;
    }
    r.area = __ldcg(a.area + u);
    if (G == 2 || G == 4)
        for (int d = 0; d < 3; d++) r.s1[d] = s1_used(a, d) ? __ldcg(a.s1[d] + u) : 0ull;
    if (G == 4)
        for (int d = 0; d < 6; d++) r.s2[d] = s2_used(a, d) ? __ldcg(a.s2[d] + u) : 0ull;
    if (G == 3 || G == 4)
        for (int d = 0; d < 5; d++) r.gw[d] = gw_used(a, d) ? __ldcg((unsigned long long *)a.gw[d] + u) : 0ull;
}

// q's own contributions plus the carried record of its only child, stored as q's
// complete record (nobody else writes q: its one child is this walker)
template <int G, bool EXACT>
__device__ __forceinline__ void rec_absorb_store(const AttrBufs &a, int q, Rec<G, EXACT> &r)
{
    if (G == 1) {  // load, combine and store the interleaved record whole; pending is cleared
        uint4 *rp = (uint4 *)(a.area + q);
        const uint4 q0 = __ldcg(rp), q1 = __ldcg(rp + 1);
        r.area += q0.x;
        r.bmin[0] = min(r.bmin[0], q0.z);
        r.bmin[1] = min(r.bmin[1], q0.w);
        r.bmin[2] = min(r.bmin[2], q1.x);
        r.bmax[0] = max(r.bmax[0], q1.y);
        r.bmax[1] = max(r.bmax[1], q1.z);
        r.bmax[2] = max(r.bmax[2], q1.w);
        __stcg(rp, make_uint4(r.area, 0u, r.bmin[0], r.bmin[1]));
        __stcg(rp + 1, make_uint4(r.bmin[2], r.bmax[0], r.bmax[1], r.bmax[2]));
        return;
    }
    r.area += __ldcg(a.area + q);
    __stcg(a.area + q, r.area);
    if (G == 1)
        for (int d = 0; d < (a.has_z ? 3 : 2); d++) {
            r.bmin[d] = min(r.bmin[d], __ldcg(a.bmin[d] + q));
            r.bmax[d] = max(r.bmax[d], __ldcg(a.bmax[d] + q));
            __stcg(a.bmin[d] + q, r.bmin[d]);
            __stcg(a.bmax[d] + q, r.bmax[d]);
        }
    if (G == 2 || G == 4)
        for (int d = 0; d < 3; d++)
            if (s1_used(a, d)) {
                r.s1[d] += __ldcg(a.s1[d] + q);
                __stcg(a.s1[d] + q, r.s1[d]);
            }
    if (G == 4)
        for (int d = 0; d < 6; d++)
            if (s2_used(a, d)) {
                r.s2[d] += __ldcg(a.s2[d] + q);
                __stcg(a.s2[d] + q, r.s2[d]);
            }
    if (G == 3 || G == 4)
        for (int d = 0; d < 5; d++) {
            if (!gw_used(a, d)) continue;
            unsigned long long *f = (unsigned long long *)a.gw[d] + q;
            if (EXACT) r.gw[d] += __ldcg(f);
            else r.gw[d] = __double_as_longlong(__longlong_as_double(r.gw[d]) + __longlong_as_double(__ldcg(f)));
            __stcg(f, r.gw[d]);
        }
}

// the carried record added into q with atomics (q has other children)
template <int G, bool EXACT>
__device__ __forceinline__ void rec_fold(const AttrBufs &a, int q, const Rec<G, EXACT> &r)
{
    atomicAdd(a.area + q, r.area);
    if (G == 1)
        for (int d = 0; d < (a.has_z ? 3 : 2); d++) {
            atomicMin(a.bmin[d] + q, r.bmin[d]);
            atomicMax(a.bmax[d] + q, r.bmax[d]);
        }
    if (G == 2 || G == 4)
        for (int d = 0; d < 3; d++)
            if (s1_used(a, d)) atomicAdd(a.s1[d] + q, r.s1[d]);
    if (G == 4)
        for (int d = 0; d < 6; d++)
            if (s2_used(a, d)) atomicAdd(a.s2[d] + q, r.s2[d]);
    if (G == 3 || G == 4)
        for (int d = 0; d < 5; d++) {
            if (!gw_used(a, d)) continue;
            if (EXACT) atomicAdd((unsigned long long *)a.gw[d] + q, r.gw[d]);
            else atomicAdd((double *)a.gw[d] + q, __longlong_as_double(r.gw[d]));
        }
}

constexpr int STALLED = -3;         // pending value of a complete node not folded upward

// Bottom-up fold limited to up_steps nodes per walker, starting at the leaves and
// carrying the current node's complete record in registers.  Into a parent with one
// child the walker adds its record and stores the parent's total directly (no
// atomics, no fences, the parent's count cleared); into a parent with several
// children it folds with atomics, and the last child to arrive (pending count)
// continues with the parent's record.  A walker stopping at a complete node marks
// it STALLED instead of folding it into its parent.  What is left (STALLED nodes and
// nodes still waiting for children) lies near the root and is finished by pointer
// jumping (k_jump_fold).
template <int G, bool EXACT>
__global__ void k_attr_up(const int *__restrict__ nodes, const unsigned long long *num_nodes,
                          const int *__restrict__ parent, AttrBufs a, int up_steps, unsigned *err)
{
    NODE_LOOP(p, nodes, num_nodes)
    {
        if (__ldcg(a.pending + p) != -1) continue;
        int u = p;
        Rec<G, EXACT> r;
        rec_load<G, EXACT>(a, u, r);
        if constexpr (G == 1) {
            // The extent record is one 32-byte sector, so each step reads everything it
            // may need at the parent q at once -- the single-child flag, q's record and
            // q's own parent (the next step's q) -- instead of one after the other: a
            // single-child step, the common one along chains, costs one round trip.
            // Only this walker writes a single-child parent; a parent with more
            // children takes the atomics below and ignores the record read early.
            int q = parent[u];
            for (int step = 0; q != NONE; step++) {
                if (step == up_steps) {
                    a.pending[u] = STALLED;
                    break;
                }
                const unsigned char sq = a.single[q];
                uint4 *rp = (uint4 *)(a.area + q);
                const uint4 q0 = __ldcg(rp), q1 = __ldcg(rp + 1);
                const int qq = parent[q];
                if (sq) {
                    r.area += q0.x;
                    r.bmin[0] = min(r.bmin[0], q0.z);
                    r.bmin[1] = min(r.bmin[1], q0.w);
                    r.bmin[2] = min(r.bmin[2], q1.x);
                    r.bmax[0] = max(r.bmax[0], q1.y);
                    r.bmax[1] = max(r.bmax[1], q1.z);
                    r.bmax[2] = max(r.bmax[2], q1.w);
                    __stcg(rp, make_uint4(r.area, 0u, r.bmin[0], r.bmin[1]));  // pending cleared
                    __stcg(rp + 1, make_uint4(r.bmin[2], r.bmax[0], r.bmax[1], r.bmax[2]));
                    u = q;
                    q = qq;
                    continue;
                }
                rec_fold<G, EXACT>(a, q, r);
                __threadfence();
                const int before = atomicSub(a.pending + q, 1);
                if (before != 1) break;
                __threadfence();
                u = q;
                q = qq;
                rec_load<G, EXACT>(a, u, r);
            }
            continue;
        }
        for (int step = 0;; step++) {
            const int q = parent[u];
            if (q == NONE) break;
            if (step == up_steps) {
                a.pending[u] = STALLED;
                break;
            }
            if (a.single[q]) {
                rec_absorb_store<G, EXACT>(a, q, r);
                a.pending[q] = 0;
                u = q;
                continue;
            }
            rec_fold<G, EXACT>(a, q, r);
            __threadfence();
            const int before = atomicSub(a.pending + q, 1);
            if (before != 1) break;
            __threadfence();
            u = q;
            rec_load<G, EXACT>(a, u, r);
        }
    }
}

// nodes left for the pointer-jumping phase, listed in any order
// (list entries beyond cap are dropped and flagged: the caller sized the list)
__global__ void k_collect_rest(const int *__restrict__ nodes, const unsigned long long *num_nodes, Field<int> pending,
                               int *list, unsigned *count, unsigned cap, unsigned *err)
{
    NODE_LOOP(p, nodes, num_nodes)
    {
        int s = pending[p];
        if (s > 0 || s == STALLED) {
            unsigned i = atomicAdd(count, 1u);
            if (list) {
                if (i < cap) list[i] = (int)p;
                else raise_error(err, DEVERR_CAPACITY);
            }
        }
    }
}

__device__ __forceinline__ unsigned rest_count(const unsigned *count, unsigned cap)
{
    const unsigned c = *count;
    return c < cap ? c : cap;
}

// Compact records of the remaining nodes: R-long arrays, one per field.
struct RestRecs {
    uint32_t *area;
    uint32_t *bmin[3], *bmax[3];
    unsigned long long *s1[3], *s2[6];
    void *gw[5];
};

template <int G>
__device__ __forceinline__ void rest_copy(const RestRecs &dst, int i, const AttrBufs &src, int u, bool to_rest)
{
    if (to_rest) {
        dst.area[i] = src.area[u];
        if (G == 1) for (int d = 0; d < 3; d++) { dst.bmin[d][i] = src.bmin[d][u]; dst.bmax[d][i] = src.bmax[d][u]; }
        if (G == 2 || G == 4) for (int d = 0; d < 3; d++) if (s1_used(src, d)) dst.s1[d][i] = src.s1[d][u];
        if (G == 4) for (int d = 0; d < 6; d++) if (s2_used(src, d)) dst.s2[d][i] = src.s2[d][u];
        if (G == 3 || G == 4)
            for (int d = 0; d < 5; d++)
                if (gw_used(src, d))
                    ((unsigned long long *)dst.gw[d])[i] = ((const unsigned long long *)src.gw[d])[u];
    } else {
        src.area[u] = dst.area[i];
        if (G == 1) for (int d = 0; d < 3; d++) { src.bmin[d][u] = dst.bmin[d][i]; src.bmax[d][u] = dst.bmax[d][i]; }
        if (G == 2 || G == 4) for (int d = 0; d < 3; d++) if (s1_used(src, d)) src.s1[d][u] = dst.s1[d][i];
        if (G == 4) for (int d = 0; d < 6; d++) if (s2_used(src, d)) src.s2[d][u] = dst.s2[d][i];
        if (G == 3 || G == 4)
            for (int d = 0; d < 5; d++)
                if (gw_used(src, d))
                    ((unsigned long long *)src.gw[d])[u] = ((const unsigned long long *)dst.gw[d])[i];
    }
}

template <int G>
__global__ void k_rest_gather(const int *__restrict__ list, const unsigned *count, unsigned cap,
                              const int *__restrict__ parent, Field<int> pending, AttrBufs a, RestRecs r, int *jump,
                              unsigned *err)
{
    const unsigned R = rest_count(count, cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        rest_copy<G>(r, (int)i, a, list[i], true);
        pending[list[i]] = -(int)(i + 16);  // position of the node in the compact list
    }
}

template <int G>
__global__ void k_rest_links(const int *__restrict__ list, const unsigned *count, unsigned cap,
                             const int *__restrict__ parent, Field<int> pending, int *jump, unsigned *err)
{
    const unsigned R = rest_count(count, cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        int q = parent[list[i]];
        int j = NONE;
        if (q != NONE) {
            int s = pending[q];
            if (s <= -16) j = -s - 16;
            else raise_error(err, DEVERR_WALK_BOUND);  // a parent of a remaining node must remain
        }
        jump[i] = j;
    }
}

// One pointer-jumping round over the remaining forest: every node adds its partial
// record into the node 2^k levels above it (sums; min/max for the bounding box).
// Reads the `in` buffers, writes `out` (initialised as a copy of `in`).
template <int G, bool EXACT>
__global__ void k_jump_fold(const unsigned *count, unsigned cap, const int *__restrict__ jin, int *jout, RestRecs in,
                            RestRecs out, AttrBufs a, const unsigned *act, unsigned *act_next)
{
    if (*act == 0) return;  // an earlier round found no jump left
    const bool has_z = a.has_z;
    const unsigned R = rest_count(count, cap);
    bool more = false;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        int j = jin[i];
        if (j == NONE) {
            jout[i] = NONE;
            continue;
        }
        jout[i] = jin[j];
        more |= jin[j] != NONE;
        atomicAdd(out.area + j, in.area[i]);
        if (G == 1)
            for (int d = 0; d < (has_z ? 3 : 2); d++) {
                atomicMin(out.bmin[d] + j, in.bmin[d][i]);
                atomicMax(out.bmax[d] + j, in.bmax[d][i]);
            }
        if (G == 2 || G == 4) for (int d = 0; d < 3; d++) if (s1_used(a, d)) atomicAdd(out.s1[d] + j, in.s1[d][i]);
        if (G == 4) for (int d = 0; d < 6; d++) if (s2_used(a, d)) atomicAdd(out.s2[d] + j, in.s2[d][i]);
        if (G == 3 || G == 4)
            for (int d = 0; d < 5; d++) {
                if (!gw_used(a, d)) continue;
                if (EXACT) atomicAdd((unsigned long long *)out.gw[d] + j, ((const unsigned long long *)in.gw[d])[i]);
                else atomicAdd((double *)out.gw[d] + j, ((const double *)in.gw[d])[i]);
            }
    }
    if (__any_sync(0xffffffffu, more) && (threadIdx.x & 31) == 0) *act_next = 1u;
}

// active rounds form a prefix; after an odd number of them the records are in r1
template <int G>
__global__ void k_rest_scatter(const int *__restrict__ list, const unsigned *count, unsigned cap, AttrBufs a,
                               RestRecs r0, RestRecs r1, const unsigned *act, int rounds)
{
    int done = 0;
    while (done < rounds && act[done]) done++;
    const RestRecs &r = (done & 1) ? r1 : r0;
    const unsigned R = rest_count(count, cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x)
        rest_copy<G>(r, (int)i, a, list[i], false);
}

// out = in over the first min(count, cap) records (device-side length)
template <int G>
__global__ void k_copy_recs(const unsigned *count, unsigned cap, RestRecs in, RestRecs out, AttrBufs a,
                            const unsigned *act)
{
    if (*act == 0) return;
    const unsigned R = rest_count(count, cap);
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        out.area[i] = in.area[i];
        if (G == 1) for (int d = 0; d < 3; d++) { out.bmin[d][i] = in.bmin[d][i]; out.bmax[d][i] = in.bmax[d][i]; }
        if (G == 2 || G == 4) for (int d = 0; d < 3; d++) if (s1_used(a, d)) out.s1[d][i] = in.s1[d][i];
        if (G == 4) for (int d = 0; d < 6; d++) if (s2_used(a, d)) out.s2[d][i] = in.s2[d][i];
        if (G == 3 || G == 4)
            for (int d = 0; d < 5; d++)
                if (gw_used(a, d)) ((unsigned long long *)out.gw[d])[i] = ((const unsigned long long *)in.gw[d])[i];
    }
}

static size_t rest_record_bytes(int group)
{
    size_t b = 4;
    if (group == 1) b += 24;
    if (group == 2) b += 24;
    if (group == 3) b += 40;
    if (group == 4) b += 24 + 48 + 40;
    return b;
}

size_t attr_rest_bytes(int group, size_t R)
{
    // list + 2 jump arrays + 2 compact record buffers (each array 256-byte aligned)
    // + the rounds' activity flags
    return 3 * ((4 * R + 255) / 256 * 256) + 2 * (rest_record_bytes(group) * R + 16 * 256) + 2 * 256;
}

static RestRecs carve(char *&m, int group, size_t R)
{
    RestRecs r{};
    auto take = [&](size_t bytes) { void *p = m; m += (bytes * R + 255) / 256 * 256; return p; };
    r.area = (uint32_t *)take(4);
    if (group == 1) for (int d = 0; d < 3; d++) { r.bmin[d] = (uint32_t *)take(4); r.bmax[d] = (uint32_t *)take(4); }
    if (group == 2 || group == 4) for (int d = 0; d < 3; d++) r.s1[d] = (unsigned long long *)take(8);
    if (group == 4) for (int d = 0; d < 6; d++) r.s2[d] = (unsigned long long *)take(8);
    if (group == 3 || group == 4) for (int d = 0; d < 5; d++) r.gw[d] = take(8);
    return r;
}

#define DCF_GROUP_SWITCH(M)                                  \
    switch (a.group * 2 + (a.exact_g ? 1 : 0)) {             \
    case 0: case 1: M(0, false); break;                      \
    case 2: case 3: M(1, false); break;                      \
    case 4: case 5: M(2, false); break;                      \
    case 6: M(3, false); break;                              \
    case 7: M(3, true); break;                               \
    case 8: M(4, false); break;                              \
    default: M(4, true); break;                              \
    }

void launch_attributes_up(const TreeView &t, AttrBufs &a, unsigned *count, int up_steps, unsigned *err, int sm,
                          cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    prof_begin(P_ATTR_UP, s);
    k_mark_leaves<<<nb, 256, 0, s>>>(t.nodes, t.num_nodes, a.pending, a.single); note_launch();
#define DCF_UP(G, E) k_attr_up<G, E><<<nb, 256, 0, s>>>(t.nodes, t.num_nodes, t.parent, a, up_steps, err); note_launch()
    DCF_GROUP_SWITCH(DCF_UP)
#undef DCF_UP
    cudaMemsetAsync(count, 0, sizeof(unsigned), s);
    k_collect_rest<<<nb, 256, 0, s>>>(t.nodes, t.num_nodes, a.pending, nullptr, count, 0u, err); note_launch();
    prof_end(P_ATTR_UP, s);
}

void launch_attributes(const TreeView &t, AttrBufs &a, unsigned *count, int up_steps, unsigned *err, int sm,
                       cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
#define DCF_PIX(G, E) k_attr_pixels<G, E><<<nb, 256, 0, s>>>(t.gval, t.g, t.parent, t.isroot, a); note_launch()
    prof_begin(P_ATTR_PIX, s);
    if (t.g.D == 1 && a.group <= 1 && agg_enabled()) {
        const int ntx = (t.g.W + AGG_T - 1) / AGG_T, nty = (t.g.H + AGG_T - 1) / AGG_T;
        if (a.group == 1) {
            static bool attr_set = false;  // opt in to more than 48 KB of dynamic shared memory, once
            if (!attr_set) {
                cudaFuncSetAttribute(k_attr_pixels_tiled<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)agg_smem_bytes<1>());
                attr_set = true;
            }
            k_attr_pixels_tiled<1><<<ntx * nty, AGG_THREADS, agg_smem_bytes<1>(), s>>>(t.g, t.parent, t.isroot, a,
                                                                                      ntx);
        } else {
            k_attr_pixels_tiled<0><<<ntx * nty, AGG_THREADS, agg_smem_bytes<0>(), s>>>(t.g, t.parent, t.isroot, a,
                                                                                      ntx);
        }
        note_launch();
    } else {
        DCF_GROUP_SWITCH(DCF_PIX)
    }
#undef DCF_PIX
    prof_end(P_ATTR_PIX, s);
    launch_attributes_up(t, a, count, up_steps, err, sm, s);
}

// Pointer-jumping phase over the nodes the walkers left.  `cap` sizes the scratch
// (exact == true: the count the caller read back; false: a capacity, the count
// staying on the device).  Enough rounds are launched for a chain of cap nodes, but
// each round flags whether any jump is left: once none is, the remaining rounds
// return at once (the forest is usually far shallower than its node count).
template <int G, bool E>
static void rest_phase(const TreeView &t, AttrBufs &a, unsigned cap, bool, unsigned *count, void *scratch,
                       unsigned *err, int sm, cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    char *m = (char *)scratch;
    int *list = (int *)m;
    m += (4 * (size_t)cap + 255) / 256 * 256;
    int *j0 = (int *)m;
    m += (4 * (size_t)cap + 255) / 256 * 256;
    int *j1 = (int *)m;
    m += (4 * (size_t)cap + 255) / 256 * 256;
    RestRecs r0 = carve(m, a.group, cap), r1 = carve(m, a.group, cap);
    unsigned *act = (unsigned *)m;  // act[k] != 0: round k has work (at most 32 rounds)
    cudaMemsetAsync(act, 0, 33 * sizeof(unsigned), s);
    cudaMemsetAsync(act, 1, 1, s);
    cudaMemsetAsync(count, 0, sizeof(unsigned), s);
    k_collect_rest<<<nb, 256, 0, s>>>(t.nodes, t.num_nodes, a.pending, list, count, cap, err); note_launch();
    if (cap == 0) return;
    const int rb = grid_for(cap, 256, sm);
    k_rest_gather<G><<<rb, 256, 0, s>>>(list, count, cap, t.parent, a.pending, a, r0, j0, err); note_launch();
    k_rest_links<G><<<rb, 256, 0, s>>>(list, count, cap, t.parent, a.pending, j0, err); note_launch();
    int rounds = 0;
    while ((1u << rounds) < cap && rounds < 31) rounds++;
    RestRecs *ri = &r0, *ro = &r1;
    int *ji = j0, *jo = j1;
    for (int k = 0; k < rounds; k++) {
        k_copy_recs<G><<<rb, 256, 0, s>>>(count, cap, *ri, *ro, a, act + k); note_launch();
        k_jump_fold<G, E><<<rb, 256, 0, s>>>(count, cap, ji, jo, *ri, *ro, a, act + k, act + k + 1); note_launch();
        RestRecs *tr = ri; ri = ro; ro = tr;
        int *tj = ji; ji = jo; jo = tj;
    }
    k_rest_scatter<G><<<rb, 256, 0, s>>>(list, count, cap, a, r0, r1, act, rounds); note_launch();
}

// Phase 2: R = number of nodes the walkers left (read back by the caller), scratch
// = attr_rest_bytes(group, R) bytes.
void launch_attributes_rest(const TreeView &t, AttrBufs &a, unsigned R, unsigned *count, void *scratch,
                            unsigned *err, int sm, cudaStream_t s)
{
    prof_begin(P_ATTR_REST, s);
#define DCF_REST(G, E) rest_phase<G, E>(t, a, R, true, count, scratch, err, sm, s)
    DCF_GROUP_SWITCH(DCF_REST)
#undef DCF_REST
    prof_end(P_ATTR_REST, s);
}

void launch_attributes_rest_cap(const TreeView &t, AttrBufs &a, unsigned cap, unsigned *count, void *scratch,
                                unsigned *err, int sm, cudaStream_t s)
{
    prof_begin(P_ATTR_REST, s);
#define DCF_REST(G, E) rest_phase<G, E>(t, a, cap, false, count, scratch, err, sm, s)
    DCF_GROUP_SWITCH(DCF_REST)
#undef DCF_REST
    prof_end(P_ATTR_REST, s);
}

__global__ void k_node_attr(Geom g, const unsigned char *__restrict__ isroot, AttrBufs a, int attr, bool area,
                            float pd0, float pd1, float pd2, double *out)
{
    const float pd[3] = {pd0, pd1, pd2};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N;
         p += (long long)gridDim.x * blockDim.x) {
        out[p] = isroot[p] ? (area ? area_value(a, (int)p, pd)
                                   : attr >= INERTIA_COL0 ? inertia_column(a, attr - INERTIA_COL0, (int)p, pd)
                                                          : attr_value(a, attr, (int)p, pd))
                           : __longlong_as_double(0x7ff8000000000000LL);
    }
}

void launch_node_attr(const TreeView &t, const AttrBufs &a, int attr, bool area, double *out, int sm,
                      cudaStream_t s)
{
    int nb = grid_for(t.g.N, 256, sm);
    k_node_attr<<<nb, 256, 0, s>>>(t.g, t.isroot, a, attr, area, t.pixdim[0], t.pixdim[1], t.pixdim[2], out); note_launch();
}

}  // namespace dcf
