// Tree construction kernels (the reference's build_local_tree_generic,
// flood.c:58-172, and its distributed correction, boundary.c:1712, re-designed for
// one GPU):
//
//   k_stats        min / max / NaN scan of the input (preprocessing.c:7-30).
//   k_tile_build   one CTA builds the max-tree of one tile in shared memory: a 1-D
//                  stack pass per row, then the rows are merged band by band with the
//                  lock-free connect() on 64-bit shared-memory node words; the tile's
//                  forest goes to the HBM node array in level-root form.
//   k_seam_merge   every edge that crosses a tile boundary is merged with connect()
//                  on the HBM node array (64-bit CAS): the on-device replacement of
//                  the MPI boundary-tree exchange and merge.
//   k_canon        flatten to the reference's canonical form (flood.c:127-141,
//                  get_levelroot :693-712) into the int32 parent array: pixel ->
//                  level root, root -> parent's level root; root flags; node count.
#include "dcf_kernels.cuh"

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

// ---------------------------------------------------------------------------
// tile build
// ---------------------------------------------------------------------------
struct SmemAcc {
    unsigned long long *w;
    unsigned *err;
    int npix;
    __device__ uint64_t load(int i) const { return ((volatile unsigned long long *)w)[i]; }
    __device__ void store(int i, uint64_t v) { ((volatile unsigned long long *)w)[i] = v; }
    __device__ bool cas(int i, uint64_t expect, uint64_t v) { return atomicCAS(w + i, expect, v) == expect; }
    __device__ long long walk_bound() const { return npix + 1; }
    __device__ void error(unsigned bit) { raise_error(err, bit); }
};

// Max-tree of one tile by the whole CTA.  The tile starts at (x0, y0, z0) of an
// image of geometry g whose pixel (x, y, z) has global index off + z*WH + y*W + x
// (off > 0 for one cutout of a batch).  smem holds tw*th*td node words followed by
// the row stacks.  Writes gval and the tile forest (level-root form, global
// indices) into gnode.
template <typename T, bool MIN>
__device__ __forceinline__ void build_tile(const T *__restrict__ img, long long off, const Geom &g, int x0, int y0,
                                           int z0, float gmax, float *__restrict__ gval,
                                           unsigned long long *__restrict__ gnode, unsigned *err,
                                           unsigned long long *smem_tile)
{
    // tile extents from the geometry (at most 4096 pixels: local indices < 2^16)
    const bool is3d = g.D > 1;
    const int TW = g.tw, TH = g.th, TD = g.td, TILE_PIX = TW * TH * TD;
    unsigned long long *snode = smem_tile;                               // TILE_PIX words
    unsigned short *sstk = (unsigned short *)(smem_tile + TILE_PIX);     // one TW-long stack per row
    const int wl = min(TW, g.W - x0), hl = min(TH, g.H - y0), dl = min(TD, g.D - z0);
    const int tid = threadIdx.x;

    for (int i = tid; i < TILE_PIX; i += TILE_THREADS) {
        int lx = i % TW, ly = (i / TW) % TH, lz = i / (TW * TH);
        uint32_t k = 0;
        if (lx < wl && ly < hl && lz < dl) {
            long long gp = off + (long long)(z0 + lz) * g.WH + (long long)(y0 + ly) * g.W + (x0 + lx);
            float lv = level_of<T, MIN>(img[gp], gmax);
            gval[gp] = lv;
            k = order_key(lv);
        }
        snode[i] = wmake(k, NONE);
    }
    __syncthreads();

    // 1-D max-tree of each row with a stack (pop higher keys; the popped chain
    // hangs off the next popped element, the last one off the new pixel).
    const int nrows = TH * TD;
    for (int r = tid; r < nrows; r += TILE_THREADS) {
        int ly = r % TH, lz = r / TH;
        if (ly >= hl || lz >= dl) continue;
        unsigned short *stk = sstk + r * TW;
        int sp = 0;
        const int base = r * TW;
        for (int lx = 0; lx < wl; lx++) {
            int i = base + lx;
            uint32_t ki = wkey(snode[i]);
            int last = NONE;
            while (sp > 0 && wkey(snode[stk[sp - 1]]) > ki) {
                int t = stk[--sp];
                if (last != NONE) snode[last] = wmake(wkey(snode[last]), t);
                last = t;
            }
            if (last != NONE) snode[last] = wmake(wkey(snode[last]), i);
            stk[sp++] = (unsigned short)i;
        }
        for (int j = sp - 1; j >= 1; j--) snode[stk[j]] = wmake(wkey(snode[stk[j]]), stk[j - 1]);
    }
    __syncthreads();

    SmemAcc acc{snode, err, TILE_PIX};
    const Offs offs = forward_offsets(g.conn);
    // merge row bands along y (each z slice), then slabs along z; at level k the
    // seams are the rows (slices) c with c % 2^(k+1) == 2^k
    for (int axis = 1; axis <= (is3d ? 2 : 1); axis++) {
        const int ext = axis == 1 ? TH : TD;
        for (int half = 1; half < ext; half <<= 1) {
            const int nseams = (ext + 2 * half - 1) / (2 * half);
            const int other = axis == 1 ? TD : TH;  // slices (axis y) or rows (axis z)
            // all edges across the seams of this level at once; correctness does not
            // depend on the order (see connect)
            const long long work = (long long)nseams * other * TW;
            for (long long w = tid; w < work; w += TILE_THREADS) {
                int lx = (int)(w % TW);
                long long rest = w / TW;
                int o = (int)(rest % other);
                int s = (int)(rest / other);
                int c = s * 2 * half + half;  // seam coordinate on the axis
                int ly, lz;
                if (axis == 1) { ly = c; lz = o; }
                else { lz = c; ly = o; }
                if (lx >= wl || ly >= hl || lz >= dl) continue;
                int p = lx + ly * TW + lz * TW * TH;
                // edges from p to the previous row / slice: the reversed forward offsets
                for (int e = 0; e < offs.n; e++) {
                    int dx = offs.d[e][0], dy = offs.d[e][1], dz = offs.d[e][2];
                    bool crosses = axis == 1 ? (dz == 0 && dy == 1) : (dz == 1);
                    if (!crosses) continue;
                    int qx = lx - dx, qy = ly - dy, qz = lz - dz;
                    if (qx < 0 || qx >= wl || qy < 0 || qy >= hl || qz < 0 || qz >= dl) continue;
                    connect(acc, p, qx + qy * TW + qz * TW * TH, MERGE_BOUND_SMEM);
                }
            }
            // levels are ordered for shorter merge walks, not for correctness:
            // without the barrier warps run ahead into the next level
            if (g.level_sync) __syncthreads();
        }
    }
    __syncthreads();

    // level-root form inside the tile (read-only walks, then each pixel writes its
    // own word): pixel -> level root, root -> parent's level root; to global indices
    unsigned short *sroot = sstk;  // the row stacks are no longer needed
    for (int i = tid; i < TILE_PIX; i += TILE_THREADS) {
        int lx = i % TW, ly = (i / TW) % TH, lz = i / (TW * TH);
        sroot[i] = (lx < wl && ly < hl && lz < dl) ? (unsigned short)levelroot_ro(acc, i) : (unsigned short)0xFFFFu;
    }
    __syncthreads();
    for (int i = tid; i < TILE_PIX; i += TILE_THREADS) {
        int lx = i % TW, ly = (i / TW) % TH, lz = i / (TW * TH);
        if (lx >= wl || ly >= hl || lz >= dl) continue;
        const uint64_t w = snode[i];
        int p = sroot[i];
        if (p == i) {  // level root: its parent node's level root
            const int q = wpar(w);
            p = q == NONE ? NONE : (int)sroot[q];
        }
        int out = NONE;
        if (p != NONE) {
            int px = p % TW, py = (p / TW) % TH, pz = p / (TW * TH);
            out = (int)(off + (long long)(z0 + pz) * g.WH + (long long)(y0 + py) * g.W + (x0 + px));
        }
        long long gp = off + (long long)(z0 + lz) * g.WH + (long long)(y0 + ly) * g.W + (x0 + lx);
        gnode[gp] = wmake(wkey(w), out);
    }
}

template <typename T, bool MIN>
__global__ void __launch_bounds__(TILE_THREADS)
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
struct GlobalAcc {
    unsigned long long *w;
    unsigned *err;
    long long n;
    __device__ uint64_t load(int i) const { return ((volatile unsigned long long *)w)[i]; }
    __device__ void store(int i, uint64_t v) { ((volatile unsigned long long *)w)[i] = v; }
    __device__ bool cas(int i, uint64_t expect, uint64_t v) { return atomicCAS(w + i, expect, v) == expect; }
    __device__ long long walk_bound() const { return n + 1; }
    __device__ void error(unsigned bit) { raise_error(err, bit); }
};

// Seam merge: work item = (tile, face, segment).  Faces are the tile's +x, -x, +y,
// -y, +z sides (forward offsets never point to -z); a segment is a run of face
// pixels one thread walks in order, merging every forward edge of each pixel that
// leaves the tile.  Every cross-tile edge leaves its low endpoint's tile through
// one of these faces, so all are merged (edges at tile corners possibly twice,
// which is harmless).
constexpr int SEAM_SEG = 4;

// largest tile face in SEAM_SEG runs
__host__ __device__ inline int seam_segments_per_face(const Geom &g)
{
    int f = g.th * g.td;
    f = f > g.tw * g.td ? f : g.tw * g.td;
    if (g.D > 1) f = f > g.tw * g.th ? f : g.tw * g.th;
    return (f + SEAM_SEG - 1) / SEAM_SEG;
}

__global__ void k_seam_merge(unsigned long long *gnode, Geom g, int ntx, int nty, int ntz, unsigned *err)
{
    const bool is3d = g.D > 1;
    const int TW = g.tw, TH = g.th, TD = g.td;
    GlobalAcc acc{gnode, err, g.N};
    const Offs offs = forward_offsets(g.conn);
    bool neg_x = false, neg_y = false;
    for (int e = 0; e < offs.n; e++) {
        neg_x |= offs.d[e][0] < 0;
        neg_y |= offs.d[e][1] < 0;
    }
    // face f: 0 +x, 1 -x, 2 +y, 3 -y, 4 +z; pixels per face and segments per face
    const int fpix[5] = {TH * TD, TH * TD, TW * TD, TW * TD, TW * TH};
    const int nseg_face = seam_segments_per_face(g);
    const long long ntiles = (long long)ntx * nty * ntz;
    const long long work = ntiles * 5 * nseg_face;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < work;
         w += (long long)gridDim.x * blockDim.x) {
        const int sg = (int)(w % nseg_face);
        const int f = (int)((w / nseg_face) % 5);
        const long long tile = w / (5LL * nseg_face);
        if ((f == 1 && !neg_x) || (f == 3 && !neg_y) || (f == 4 && !is3d)) continue;
        if (sg * SEAM_SEG >= fpix[f]) continue;
        const int tx = (int)(tile % ntx), ty = (int)((tile / ntx) % nty), tz = (int)(tile / ((long long)ntx * nty));
        const int x0 = tx * TW, y0 = ty * TH, z0 = tz * TD;
        const int wl = min(TW, g.W - x0), hl = min(TH, g.H - y0), dl = min(TD, g.D - z0);
        for (int k = sg * SEAM_SEG; k < min(fpix[f], (sg + 1) * SEAM_SEG); k++) {
            int lx, ly, lz;
            if (f <= 1) { lx = f == 0 ? wl - 1 : 0; ly = k % TH; lz = k / TH; }
            else if (f <= 3) { ly = f == 2 ? hl - 1 : 0; lx = k % TW; lz = k / TW; }
            else { lz = dl - 1; lx = k % TW; ly = k / TW; }
            if (lx >= wl || ly >= hl || lz >= dl) continue;
            const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
            const int p = (int)((long long)z * g.WH + (long long)y * g.W + x);
            for (int e = 0; e < offs.n; e++) {
                int qx = x + offs.d[e][0], qy = y + offs.d[e][1], qz = z + offs.d[e][2];
                if (qx < 0 || qx >= g.W || qy < 0 || qy >= g.H || qz >= g.D) continue;
                if (qx >= x0 && qx < x0 + TW && qy >= y0 && qy < y0 + TH && qz >= z0 && qz < z0 + TD) continue;
                connect(acc, p, (int)((long long)qz * g.WH + (long long)qy * g.W + qx), MERGE_BOUND_GLOBAL);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// canonical form: read-only walks on the node words, each pixel writes only its
// own parent entry and root flag
// ---------------------------------------------------------------------------
__global__ void k_canon(unsigned long long *gnode, Geom g, int *parent, unsigned char *isroot,
                        unsigned long long *num_nodes, unsigned *err)
{
    GlobalAcc acc{gnode, err, g.N};
    unsigned cnt = 0;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N;
         p += (long long)gridDim.x * blockDim.x) {
        const int r = levelroot_ro(acc, (int)p);
        if (r != (int)p) {
            parent[p] = r;
            isroot[p] = 0;
        } else {
            const int q = wpar(acc.load((int)p));
            parent[p] = q == NONE ? NONE : levelroot_ro(acc, q);
            isroot[p] = 1;
            cnt++;
        }
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(num_nodes, (unsigned long long)cnt);
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
template <typename T, bool MIN>
static void build_t(const BuildArgs &a, cudaStream_t s)
{
    const T *img = (const T *)a.img;
    const int TW = a.g.tw, TH = a.g.th, TD = a.g.td;
    dim3 grid((a.g.W + TW - 1) / TW, (a.g.H + TH - 1) / TH, (a.g.D + TD - 1) / TD);
    const size_t smem = (size_t)TW * TH * TD * (8 + 2);
    prof_begin(P_TILE, s);
    k_tile_build<T, MIN><<<grid, TILE_THREADS, smem, s>>>(img, a.g, a.kmax, a.gval, a.node, a.err);
    prof_end(P_TILE, s);
    prof_begin(P_SEAM, s);
    {
        const int nseg_face = seam_segments_per_face(a.g);
        const long long work = (long long)grid.x * grid.y * grid.z * 5 * nseg_face;
        k_seam_merge<<<grid_for(work, 128, a.sm_count), 128, 0, s>>>(a.node, a.g, grid.x, grid.y, grid.z, a.err);
    }
    prof_end(P_SEAM, s);
    int nb = grid_for(a.g.N, 256, a.sm_count);
    prof_begin(P_CANON, s);
    k_canon<<<nb, 256, 0, s>>>(a.node, a.g, a.parent, a.isroot, a.num_nodes, a.err);
    prof_end(P_CANON, s);
}

void launch_stats(int dtype, const void *img, long long n, unsigned *kmin, unsigned *kmax, unsigned *nans,
                  int sm_count, cudaStream_t s)
{
    int nb = grid_for(n, 256, sm_count);
    prof_begin(P_STATS, s);
    switch (dtype) {
    case U8: k_stats<uint8_t><<<nb, 256, 0, s>>>((const uint8_t *)img, n, kmin, kmax, nans); break;
    case U16: k_stats<uint16_t><<<nb, 256, 0, s>>>((const uint16_t *)img, n, kmin, kmax, nans); break;
    case U32: k_stats<uint32_t><<<nb, 256, 0, s>>>((const uint32_t *)img, n, kmin, kmax, nans); break;
    default: k_stats<float><<<nb, 256, 0, s>>>((const float *)img, n, kmin, kmax, nans); break;
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
