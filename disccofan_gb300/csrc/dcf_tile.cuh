// Device building blocks shared by the single-image and the batched tree builds:
// the node-word accessors for shared memory (SmemAcc) and HBM (GlobalAcc) that
// connect() works through, and build_tile, the max-tree of one tile by one CTA.
#pragma once
#include "dcf_kernels.cuh"

namespace dcf {

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
// (off > 0 for one cutout of a batch).  Writes gval and the tile forest
// (level-root form, global indices) into gnode.
//
// Shared-memory layout (tile_smem_bytes): node words with a padded row stride
// RS = tw + 1 (local index of pixel (lx, ly, lz) = lx + ly*RS + lz*RS*th), then one
// stack per row with stride tw + 2 entries.  The row pass runs one row per thread
// in lock-step; unpadded strides of tw words would put all 32 rows of a warp in
// the same shared-memory bank at every step.
template <typename T, bool MIN>
__device__ __forceinline__ void build_tile(const T *__restrict__ img, long long off, const Geom &g, int x0, int y0,
                                           int z0, float gmax, float *__restrict__ gval,
                                           unsigned long long *__restrict__ gnode, unsigned *err,
                                           unsigned long long *smem_tile)
{
    // tile extents from the geometry (at most 4096 pixels: local indices < 2^16)
    const bool is3d = g.D > 1;
    const int TW = g.tw, TH = g.th, TD = g.td;
    const int RS = TW + 1, SS = TW + 2, SLICE = RS * TH, WORDS = RS * TH * TD;
    unsigned long long *snode = smem_tile;                            // WORDS node words
    unsigned short *sstk = (unsigned short *)(smem_tile + WORDS);     // one stack per row
    const int wl = min(TW, g.W - x0), hl = min(TH, g.H - y0), dl = min(TD, g.D - z0);
    const int tid = threadIdx.x;

    for (int i = tid; i < WORDS; i += TILE_THREADS) {
        int lx = i % RS, ly = (i / RS) % TH, lz = i / SLICE;
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
        unsigned short *stk = sstk + r * SS;
        int sp = 0;
        const int base = r * RS;
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

    SmemAcc acc{snode, err, WORDS};
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
                int p = lx + ly * RS + lz * SLICE;
                // edges from p to the previous row / slice: the reversed forward offsets
                for (int e = 0; e < offs.n; e++) {
                    int dx = offs.d[e][0], dy = offs.d[e][1], dz = offs.d[e][2];
                    bool crosses = axis == 1 ? (dz == 0 && dy == 1) : (dz == 1);
                    if (!crosses) continue;
                    int qx = lx - dx, qy = ly - dy, qz = lz - dz;
                    if (qx < 0 || qx >= wl || qy < 0 || qy >= hl || qz < 0 || qz >= dl) continue;
                    connect_smem(acc, p, qx + qy * RS + qz * SLICE, MERGE_BOUND_SMEM);
                }
            }
            // levels are ordered for shorter merge walks, not for correctness:
            // without the barrier warps run ahead into the next level
            if (g.level_sync) __syncthreads();
        }
    }
    __syncthreads();

    // level-root form inside the tile: pixel -> level root, root -> parent's level
    // root; to global indices.  Level roots by pointer doubling over the equal-key
    // links (a flat zone of F pixels can be a chain of ~F links, so walking it from
    // every pixel would cost O(F^2)): r(i) = parent if it has i's key, else i; then
    // r(i) = r(r(i)) until every chain (at most WORDS long) has collapsed.
    unsigned short *sroot = sstk;  // the row stacks (>= WORDS entries) are no longer needed
    for (int i = tid; i < WORDS; i += TILE_THREADS) {
        int lx = i % RS, ly = (i / RS) % TH, lz = i / SLICE;
        unsigned short r = (unsigned short)i;
        if (lx < wl && ly < hl && lz < dl) {
            const uint64_t w = snode[i];
            const int q = wpar(w);
            if (q != NONE && wkey(snode[q]) == wkey(w)) r = (unsigned short)q;
        }
        sroot[i] = r;
    }
    __syncthreads();
    for (int span = 1; span < WORDS; span <<= 1) {
        for (int i = tid; i < WORDS; i += TILE_THREADS) sroot[i] = sroot[sroot[i]];
        __syncthreads();
    }
    for (int i = tid; i < WORDS; i += TILE_THREADS) {
        int lx = i % RS, ly = (i / RS) % TH, lz = i / SLICE;
        if (lx >= wl || ly >= hl || lz >= dl) continue;
        const uint64_t w = snode[i];
        int p = sroot[i];
        if (p == i) {  // level root: its parent node's level root
            const int q = wpar(w);
            p = q == NONE ? NONE : (int)sroot[q];
        }
        int out = NONE;
        if (p != NONE) {
            int px = p % RS, py = (p / RS) % TH, pz = p / SLICE;
            out = (int)(off + (long long)(z0 + pz) * g.WH + (long long)(y0 + py) * g.W + (x0 + px));
        }
        long long gp = off + (long long)(z0 + lz) * g.WH + (long long)(y0 + ly) * g.W + (x0 + lx);
        gnode[gp] = wmake(wkey(w), out);
    }
}

// node words in HBM (seam merges)
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

// Appends one cross-tile edge (p, q) with its level min(key p, key q) to e;
// warp-aggregated counter and histogram atomics.  A warp collective: every lane
// calls it, `valid` says whether the lane has an edge.
__device__ __forceinline__ void seam_append(SeamEdges &e, const unsigned long long *gnode, bool valid, int p, int q)
{
    const int lane = threadIdx.x & 31;
    unsigned lvl = 0;
    if (valid) {
        const unsigned kp = wkey(((const volatile unsigned long long *)gnode)[p]);
        const unsigned kq = wkey(((const volatile unsigned long long *)gnode)[q]);
        lvl = kp < kq ? kp : kq;
    }
    const unsigned m = __ballot_sync(0xffffffffu, valid);
    if (!m) return;
    unsigned base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(e.count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    const unsigned bin = valid ? lvl >> 16 : 0xFFFFFFFFu;
    const unsigned same = __match_any_sync(0xffffffffu, bin);
    if (!valid) return;
    if (lane == __ffs(same) - 1) atomicAdd(e.hist + bin, (unsigned)__popc(same));
    const unsigned i = base + __popc(m & ((1u << lane) - 1u));
    if ((long long)i < e.cap) {
        e.pq[i] = make_int2(p, q);
        e.lvl[i] = lvl;
    }
}

}  // namespace dcf
