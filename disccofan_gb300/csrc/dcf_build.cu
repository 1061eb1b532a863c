// Tree construction kernels (the reference's build_local_tree_generic,
// flood.c:58-172, and its distributed correction, boundary.c:1712, re-designed for
// one GPU):
//
//   k_stats        min / max / NaN scan of the input (preprocessing.c:7-30).
//   k_tile_build   one CTA builds the max-tree of one tile in shared memory: a 1-D
//                  stack pass per row, then the rows are merged band by band with the
//                  lock-free connect() on shared-memory node words (32-bit for u8/u16,
//                  64-bit for u32/f32); the tile's forest goes to the HBM node array
//                  in level-root form (dcf_tile.cuh).
//   k_seam_collect, k_seam_bucket (or k_seam_direct)
//                  every edge that crosses a tile boundary is merged with connect()
//                  on the HBM node array (64-bit CAS): the on-device replacement of
//                  the MPI boundary-tree exchange and merge.
//   k_canon        flatten to the reference's canonical form (flood.c:127-141,
//                  get_levelroot :693-712) into the int32 parent array: pixel ->
//                  level root, root -> parent's level root; root flags.  Then the
//                  level-root list (k_nodes_count/scan/emit).
#include "dcf_tile.cuh"

namespace dcf {

// ---------------------------------------------------------------------------
// statistics
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_stats(const T *__restrict__ img, long long n, unsigned *kmin, unsigned *kmax,
                        unsigned *nan_count)
{
    unsigned lo = 0xFFFFFFFFu, hi = 0u, nans = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        float v = to_float<T>(img[i]);
        if (v != v) {
            nans++;
            continue;
        }
        unsigned k = order_key(v);
        lo = min(lo, k);
        hi = max(hi, k);
    }
    for (int o = 16; o; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        nans += __shfl_xor_sync(0xffffffffu, nans, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(kmin, lo);
        atomicMax(kmax, hi);
        if (nans) atomicAdd(nan_count, nans);
    }
}

template <typename T, bool MIN>
__global__ void __launch_bounds__(TileCfg<T>::threads, TileCfg<T>::min_blocks)
k_tile_build(const T *__restrict__ img, Geom g, const unsigned *kmax, float *__restrict__ gval,
             unsigned long long *__restrict__ gnode, unsigned *err)
{
    extern __shared__ unsigned long long smem_tile[];
    const float gmax = MIN ? key_to_level(*kmax) : 0.0f;
    build_tile<T, MIN>(img, 0, g, blockIdx.x * g.tw, blockIdx.y * g.th, blockIdx.z * g.td, gmax, gval, gnode, err,
                       smem_tile);
}

// ---------------------------------------------------------------------------
// seam merge in HBM
// ---------------------------------------------------------------------------
// Seam merge.  Work item = (tile, face, face pixel, forward offset).  Faces are the
// tile's +x, -x, +y, -y, +z sides (forward offsets never point to -z); face f takes
// the offsets that point out through it (dx = +1 for +x, ...).  Every cross-tile
// edge leaves its low endpoint's tile through at least one face it points out of,
// so all are found (corner edges possibly twice, which is harmless).  Each edge is
// one connect by one thread: on deep trees (high-dynamic-range images) a connect
// can walk a root path of 10^5 nodes, so no thread may run several in a row.
__host__ __device__ inline int seam_face_pixels(const Geom &g)
{
    int f = g.th * g.td;
    f = f > g.tw * g.td ? f : g.tw * g.td;
    if (g.D > 1) f = f > g.tw * g.th ? f : g.tw * g.th;
    return f;
}

__host__ __device__ inline long long seam_items(const Geom &g, long long ntiles)
{
    return ntiles * 5 * seam_face_pixels(g) * forward_offsets(g.conn).n;
}

// decode work item w into an edge (p, q); false if the item holds none or the edge
// is implied by others (edge_implied; keys read from the tile builds' words)
__device__ __forceinline__ bool seam_item(const Geom &g, int ntx, int nty, const Offs &offs, int fmax, long long w,
                                          const unsigned long long *gnode, int &p, int &q)
{
    const int TW = g.tw, TH = g.th, TD = g.td;
    // w = ((tile * 5 + f) * fmax + k) * offs.n + e: one 64-bit division splits off
    // the tile, the rest (below 5 * 4096 * 13) is decoded in 32 bits
    const int span = 5 * fmax * offs.n;
    const int tile = (int)(w / span);
    int r = (int)(w - (long long)tile * span);
    const int e = r % offs.n;
    r /= offs.n;
    const int k = r % fmax;
    const int f = r / fmax;
    const int dx = offs.d[e][0], dy = offs.d[e][1], dz = offs.d[e][2];
    const bool out = f == 0 ? dx > 0 : f == 1 ? dx < 0 : f == 2 ? dy > 0 : f == 3 ? dy < 0 : dz > 0;
    const int fpix = f <= 1 ? TH * TD : (f <= 3 ? TW * TD : TW * TH);
    if (!out || k >= fpix || (f == 4 && g.D == 1)) return false;
    const int tx = tile % ntx, ty = (tile / ntx) % nty, tz = tile / (ntx * nty);
    const int x0 = tx * TW, y0 = ty * TH, z0 = tz * TD;
    const int wl = min(TW, g.W - x0), hl = min(TH, g.H - y0), dl = min(TD, g.D - z0);
    int lx, ly, lz;
    if (f <= 1) { lx = f == 0 ? wl - 1 : 0; ly = k % TH; lz = k / TH; }
    else if (f <= 3) { ly = f == 2 ? hl - 1 : 0; lx = k % TW; lz = k / TW; }
    else { lz = dl - 1; lx = k % TW; ly = k / TW; }
    if (lx >= wl || ly >= hl || lz >= dl) return false;
    const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
    const int qx = x + dx, qy = y + dy, qz = z + dz;
    if (qx < 0 || qx >= g.W || qy < 0 || qy >= g.H || qz >= g.D) return false;
    p = (int)((long long)z * g.WH + (long long)y * g.W + x);
    q = (int)((long long)qz * g.WH + (long long)qy * g.W + qx);
    if (offs.n > 3) {
        const unsigned kp = wkey(gnode[p]), kq = wkey(gnode[q]);
        const int pp = p;
        auto key_at = [&](int sx, int sy, int sz) {
            return wkey(gnode[pp + (long long)sz * g.WH + (long long)sy * g.W + sx]);
        };
        if (edge_implied(dx, dy, dz, kp < kq ? kp : kq, key_at)) return false;
    }
    return true;
}

// every edge at once
__global__ void k_seam_direct(unsigned long long *gnode, Geom g, int ntx, int nty, int ntz, unsigned *err)
{
    GlobalAcc acc{gnode, err, g.N};
    const Offs offs = forward_offsets(g.conn);
    const int fmax = seam_face_pixels(g);
    const long long work = seam_items(g, (long long)ntx * nty * ntz);
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < work;
         w += (long long)gridDim.x * blockDim.x) {
        int p, q;
        if (seam_item(g, ntx, nty, offs, fmax, w, gnode, p, q)) connect(acc, p, q, merge_bound_global(g));
    }
}

__global__ void k_seam_collect(const unsigned long long *gnode, Geom g, int ntx, int nty, int ntz, SeamEdges e)
{
    const Offs offs = forward_offsets(g.conn);
    const int fmax = seam_face_pixels(g);
    const long long work = seam_items(g, (long long)ntx * nty * ntz);
    const int lane = threadIdx.x & 31;
    // warp-uniform loop: seam_append is a warp collective
    for (long long base = blockIdx.x * (long long)blockDim.x + threadIdx.x - lane; base < work;
         base += (long long)gridDim.x * blockDim.x) {
        int p = 0, q = 0;
        const bool valid = base + lane < work && seam_item(g, ntx, nty, offs, fmax, base + lane, gnode, p, q);
        seam_append(e, gnode, valid, p, q);
    }
}

long long seam_edge_bound(const Geom &g, long long ntiles)
{
    const Offs o = forward_offsets(g.conn);
    int n[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < o.n; i++) {
        n[0] += o.d[i][0] > 0;
        n[1] += o.d[i][0] < 0;
        n[2] += o.d[i][1] > 0;
        n[3] += o.d[i][1] < 0;
        n[4] += o.d[i][2] > 0;
    }
    const long long fpix[5] = {(long long)g.th * g.td, (long long)g.th * g.td, (long long)g.tw * g.td,
                               (long long)g.tw * g.td, (long long)g.tw * g.th};
    long long per = 0;
    for (int f = 0; f < 5; f++) per += fpix[f] * n[f];
    return ntiles * per;
}

static size_t al256(size_t b) { return (b + 255) / 256 * 256; }

size_t seam_edges_bytes(long long cap, int buckets)
{
    return al256(8 * (size_t)cap) * 2 + al256(4 * (size_t)cap) + al256(4 * SEAM_BINS) + al256(2 * SEAM_BINS) +
           al256(4 * (2 * (size_t)buckets + 1)) + al256(4) + 256;
}

SeamEdges seam_edges_carve(void *mem, long long cap, int buckets)
{
    SeamEdges e;
    char *m = (char *)mem;
    auto take = [&](size_t b) { void *p = m; m += al256(b); return p; };
    e.pq = (int2 *)take(8 * (size_t)cap);
    e.sorted = (int2 *)take(8 * (size_t)cap);
    e.lvl = (unsigned *)take(4 * (size_t)cap);
    e.hist = (unsigned *)take(4 * SEAM_BINS);
    e.bin_bucket = (unsigned short *)take(2 * SEAM_BINS);
    e.bstart = (unsigned *)take(4 * (2 * (size_t)buckets + 1));
    e.count = (unsigned *)take(4);
    e.cap = cap;
    e.buckets = buckets;
    return e;
}

// Bucket boundaries from the level histogram (one block): bins are assigned in
// order to buckets of about count / buckets edges; bstart[0..B] is the exclusive
// prefix of the bucket sizes, bstart[B+1..2B] the scatter counters (zeroed).
__global__ void __launch_bounds__(1024) k_seam_bounds(SeamEdges e)
{
    __shared__ unsigned s_sum[1024];
    __shared__ unsigned s_bcount[1024];
    const int t = threadIdx.x, B = e.buckets;
    const unsigned total = (long long)*e.count < e.cap ? *e.count : (unsigned)e.cap;
    const unsigned per = total / B + 1;
    constexpr int PER_T = SEAM_BINS / 1024;
    unsigned local = 0;
    for (int j = 0; j < PER_T; j++) local += e.hist[t * PER_T + j];
    s_sum[t] = local;
    s_bcount[t] = 0;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // inclusive scan
        const unsigned v = t >= o ? s_sum[t - o] : 0;
        __syncthreads();
        s_sum[t] += v;
        __syncthreads();
    }
    unsigned run = s_sum[t] - local;
    for (int j = 0; j < PER_T; j++) {
        const int bin = t * PER_T + j;
        const unsigned h = e.hist[bin];
        const unsigned b = min((unsigned)(B - 1), run / per);
        e.bin_bucket[bin] = (unsigned short)b;
        if (h) atomicAdd(s_bcount + b, h);
        run += h;
    }
    __syncthreads();
    if (t == 0) {
        unsigned acc = 0;
        for (int b = 0; b < B; b++) {
            e.bstart[b] = acc;
            acc += s_bcount[b];
            e.bstart[B + 1 + b] = 0;
        }
        e.bstart[B] = acc;
    }
}

__global__ void k_seam_scatter(SeamEdges e)
{
    const unsigned total = (long long)*e.count < e.cap ? *e.count : (unsigned)e.cap;
    const int lane = threadIdx.x & 31;
    unsigned *fill = e.bstart + e.buckets + 1;
    for (long long base = blockIdx.x * (long long)blockDim.x + threadIdx.x - lane; base < total;
         base += (long long)gridDim.x * blockDim.x) {
        const long long i = base + lane;
        const bool valid = i < total;
        const unsigned b = valid ? e.bin_bucket[e.lvl[i] >> 16] : 0xFFFFFFFFu;
        const unsigned same = __match_any_sync(0xffffffffu, b);
        if (!valid) continue;
        const int leader = __ffs(same) - 1;
        unsigned pos = 0;
        if (lane == leader) pos = atomicAdd(fill + b, (unsigned)__popc(same));
        pos = __shfl_sync(same, pos, leader);
        e.sorted[e.bstart[b] + pos + __popc(same & ((1u << lane) - 1u))] = e.pq[i];
    }
}

__global__ void k_seam_bucket(SeamEdges e, int b, unsigned long long *gnode, long long n, long long bound,
                              unsigned *err)
{
    GlobalAcc acc{gnode, err, n};
    const unsigned lo = e.bstart[b], hi = e.bstart[b + 1];
    for (long long i = lo + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < hi;
         i += (long long)gridDim.x * blockDim.x) {
        const int2 pq = e.sorted[i];
        connect(acc, pq.x, pq.y, bound);
    }
}

void launch_seam_buckets(SeamEdges &e, unsigned long long *node, long long n, long long merge_bound, unsigned *err,
                         int sm, cudaStream_t s)
{
    k_seam_bounds<<<1, 1024, 0, s>>>(e); note_launch();
    k_seam_scatter<<<grid_for(e.cap, 256, sm), 256, 0, s>>>(e); note_launch();
    const int gb = grid_for(e.cap / e.buckets + 1, 128, sm);
    for (int b = 0; b < e.buckets; b++) {
        k_seam_bucket<<<gb, 128, 0, s>>>(e, b, node, n, merge_bound > 0 ? merge_bound : MERGE_BOUND_GLOBAL, err);
        note_launch();
    }
}

// ---------------------------------------------------------------------------
// canonical form: read-only walks on the node words, each pixel writes only its
// own parent entry and root flag
// ---------------------------------------------------------------------------
// The node words are final here (no kernel writes them any more), so they are read
// through the non-coherent path and stay in L1: a pixel's parent is mostly in its
// own tile.  Each walk carries the word it loaded last, so a pixel costs its own
// word, its parent's, and the word that shows where the parent's level ends.
__global__ void k_canon(const unsigned long long *__restrict__ gnode, Geom g, int *parent, unsigned char *isroot,
                        unsigned *err)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N;
         p += (long long)gridDim.x * blockDim.x) {
        uint64_t w = __ldg(gnode + p);
        const uint32_t k = wkey(w);
        int r = (int)p, q = wpar(w);
        uint64_t wq = 0;
        long long it = 0;
        for (; q != NONE && it <= g.N; it++) {  // p's level root r; q its parent
            wq = __ldg(gnode + q);
            if (wkey(wq) != k) break;
            r = q;
            q = wpar(wq);
        }
        if (r != (int)p) {
            parent[p] = r;
            isroot[p] = 0;
        } else {
            int s = q;  // p is a level root: its parent's level root
            if (q != NONE) {
                const uint32_t kq = wkey(wq);
                for (int t = wpar(wq); t != NONE && it <= g.N; it++) {
                    const uint64_t wt = __ldg(gnode + t);
                    if (wkey(wt) != kq) break;
                    s = t;
                    t = wpar(wt);
                }
            }
            parent[p] = s;
            isroot[p] = 1;
        }
        if (it > g.N) raise_error(err, DEVERR_WALK_BOUND);
    }
}

// ---------------------------------------------------------------------------
// level-root list: the level roots in ascending index order, so that passes over
// the nodes run full warps of nodes instead of scanning every pixel (a 16384^2
// u16 max tree has one level root in 4.8 pixels, the min tree one in 18.6).
// Ordered compaction in three launches over chunks of NL_CHUNK pixels: count the
// roots of each chunk, scan the counts (one block), then write each chunk's roots
// at its offset.  Each thread takes 32 consecutive root flags.
// ---------------------------------------------------------------------------
constexpr int NL_THREADS = 256, NL_CHUNK = NL_THREADS * 32;

__host__ __device__ inline long long node_list_chunks(long long n) { return (n + NL_CHUNK - 1) / NL_CHUNK; }

size_t node_list_bytes(long long n)
{
    return (size_t)(4 * n + 255) / 256 * 256 + (size_t)(4 * node_list_chunks(n) + 255) / 256 * 256;
}

// bit j = root flag of pixel first + j (flags are 0 or 1)
__device__ __forceinline__ unsigned root_bits(const unsigned char *__restrict__ isroot, long long n, long long first)
{
    unsigned m = 0;
    if (first + 32 <= n) {  // first is a multiple of 32 and isroot 256-byte aligned
        const uint4 a = *(const uint4 *)(isroot + first), b = *(const uint4 *)(isroot + first + 16);
        const unsigned w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int k = 0; k < 8; k++) m |= (((w[k] & 0x01010101u) * 0x01020408u) >> 24) << (4 * k);
    } else {
        for (int j = 0; first + j < n; j++) m |= (unsigned)(isroot[first + j] != 0) << j;
    }
    return m;
}

// exclusive block scan of one value per thread (NL_THREADS threads); *total = sum
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *total)
{
    __shared__ unsigned warp_sum[NL_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_sum[warp] = inc;
    __syncthreads();
    unsigned before = 0, all = 0;
    for (int w = 0; w < NL_THREADS / 32; w++) {
        if (w < warp) before += warp_sum[w];
        all += warp_sum[w];
    }
    __syncthreads();  // warp_sum is reused by the next call
    *total = all;
    return before + inc - v;
}

__global__ void __launch_bounds__(NL_THREADS) k_nodes_count(const unsigned char *__restrict__ isroot, long long n,
                                                            unsigned *counts)
{
    const long long chunks = node_list_chunks(n);
    for (long long c = blockIdx.x; c < chunks; c += gridDim.x) {
        const long long first = c * NL_CHUNK + (long long)threadIdx.x * 32;
        const unsigned m = first < n ? root_bits(isroot, n, first) : 0u;
        unsigned total;
        block_excl_scan(__popc(m), &total);
        if (threadIdx.x == 0) counts[c] = total;
    }
}

// exclusive prefix of the chunk counts in place (one block of 1024 threads)
__global__ void __launch_bounds__(1024) k_nodes_scan(unsigned *counts, long long chunks,
                                                     unsigned long long *listed)
{
    __shared__ unsigned long long part[1024];
    const long long per = (chunks + 1023) / 1024;
    const long long lo = threadIdx.x * per, hi = lo + per < chunks ? lo + per : chunks;
    unsigned long long s = 0;
    for (long long i = lo; i < hi; i++) s += counts[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned long long t = threadIdx.x >= o ? part[threadIdx.x - o] : 0ull;
        __syncthreads();
        part[threadIdx.x] += t;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - s;
    for (long long i = lo; i < hi; i++) {
        const unsigned c = counts[i];
        counts[i] = (unsigned)run;
        run += c;
    }
    if (threadIdx.x == 1023 && listed) *listed = part[1023];
}

__global__ void __launch_bounds__(NL_THREADS) k_nodes_emit(const unsigned char *__restrict__ isroot, long long n,
                                                           const unsigned *__restrict__ offsets, int *nodes)
{
    const long long chunks = node_list_chunks(n);
    for (long long c = blockIdx.x; c < chunks; c += gridDim.x) {
        const long long first = c * NL_CHUNK + (long long)threadIdx.x * 32;
        unsigned m = first < n ? root_bits(isroot, n, first) : 0u;
        unsigned total;
        unsigned long long at = (unsigned long long)offsets[c] + block_excl_scan(__popc(m), &total);
        while (m) {
            const int j = __ffs(m) - 1;
            nodes[at++] = (int)(first + j);
            m &= m - 1;
        }
    }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
void launch_canon(unsigned long long *node, const Geom &g, int *parent, unsigned char *isroot,
                  unsigned long long *num_nodes, int *nodes, unsigned *err, int sm_count, cudaStream_t s)
{
    prof_begin(P_CANON, s);
    k_canon<<<grid_for(g.N, 256, sm_count), 256, 0, s>>>(node, g, parent, isroot, err); note_launch();
    const long long chunks = node_list_chunks(g.N);
    unsigned *counts = (unsigned *)((char *)nodes + (size_t)(4 * g.N + 255) / 256 * 256);
    const int nb = (int)(chunks < (long long)sm_count * 16 ? chunks : (long long)sm_count * 16);
    k_nodes_count<<<nb, NL_THREADS, 0, s>>>(isroot, g.N, counts); note_launch();
    k_nodes_scan<<<1, 1024, 0, s>>>(counts, chunks, num_nodes); note_launch();  // the node count
    k_nodes_emit<<<nb, NL_THREADS, 0, s>>>(isroot, g.N, counts, nodes); note_launch();
    prof_end(P_CANON, s);
}

template <typename T, bool MIN>
static void build_t(const BuildArgs &a, cudaStream_t s)
{
    const T *img = (const T *)a.img;
    const int TW = a.g.tw, TH = a.g.th, TD = a.g.td;
    dim3 grid((a.g.W + TW - 1) / TW, (a.g.H + TH - 1) / TH, (a.g.D + TD - 1) / TD);
    const size_t smem = tile_smem_bytes(TW, TH, TD, TileCfg<T>::word_bytes);
    // the largest shared-memory split of the SM, so the register file alone bounds
    // the resident tiles (set once per instantiation)
    static bool carveout = (cudaFuncSetAttribute(k_tile_build<T, MIN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                 cudaSharedmemCarveoutMaxShared),
                            true);
    (void)carveout;
    prof_begin(P_TILE, s);
    k_tile_build<T, MIN><<<grid, TileCfg<T>::threads, smem, s>>>(img, a.g, a.kmax, a.gval, a.node, a.err); note_launch();
    prof_end(P_TILE, s);
    prof_begin(P_SEAM, s);
    {
        const long long work = seam_items(a.g, (long long)grid.x * grid.y * grid.z);
        if (a.seam.buckets > 0) {
            SeamEdges e = a.seam;
            cudaMemsetAsync(e.count, 0, 4, s);
            cudaMemsetAsync(e.hist, 0, 4 * SEAM_BINS, s);
            k_seam_collect<<<grid_for(work, 256, a.sm_count), 256, 0, s>>>(a.node, a.g, grid.x, grid.y, grid.z, e); note_launch();
            launch_seam_buckets(e, a.node, a.g.N, a.g.merge_bound, a.err, a.sm_count, s);
        } else {
            k_seam_direct<<<grid_for(work, 128, a.sm_count), 128, 0, s>>>(a.node, a.g, grid.x, grid.y, grid.z, a.err); note_launch();
        }
    }
    prof_end(P_SEAM, s);
    launch_canon(a.node, a.g, a.parent, a.isroot, a.num_nodes, a.nodes, a.err, a.sm_count, s);
}

void launch_stats(int dtype, const void *img, long long n, unsigned *kmin, unsigned *kmax, unsigned *nans,
                  int sm_count, cudaStream_t s)
{
    int nb = grid_for(n, 256, sm_count);
    prof_begin(P_STATS, s);
    switch (dtype) {
    case U8: k_stats<uint8_t><<<nb, 256, 0, s>>>((const uint8_t *)img, n, kmin, kmax, nans); note_launch(); break;
    case U16: k_stats<uint16_t><<<nb, 256, 0, s>>>((const uint16_t *)img, n, kmin, kmax, nans); note_launch(); break;
    case U32: k_stats<uint32_t><<<nb, 256, 0, s>>>((const uint32_t *)img, n, kmin, kmax, nans); note_launch(); break;
    default: k_stats<float><<<nb, 256, 0, s>>>((const float *)img, n, kmin, kmax, nans); note_launch(); break;
    }
    prof_end(P_STATS, s);
}

void launch_build(const BuildArgs &a, cudaStream_t s)
{
    switch (a.dtype * 2 + (a.tree_min ? 1 : 0)) {
    case 0: build_t<uint8_t, false>(a, s); break;
    case 1: build_t<uint8_t, true>(a, s); break;
    case 2: build_t<uint16_t, false>(a, s); break;
    case 3: build_t<uint16_t, true>(a, s); break;
    case 4: build_t<uint32_t, false>(a, s); break;
    case 5: build_t<uint32_t, true>(a, s); break;
    case 6: build_t<float, false>(a, s); break;
    default: build_t<float, true>(a, s); break;
    }
}

}  // namespace dcf
