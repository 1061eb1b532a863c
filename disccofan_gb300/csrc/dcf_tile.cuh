// Device building blocks shared by the single-image and the batched tree builds:
// the node-word accessors for shared memory (SmemAcc) and HBM (GlobalAcc) that
// connect() works through, and build_tile, the max-tree of one tile by one CTA.
#pragma once
#include "dcf_kernels.cuh"

namespace dcf {

// ---------------------------------------------------------------------------
// tile build
// ---------------------------------------------------------------------------
// Shared-memory node words.  Word64: order key (high 32 bits) and local parent
// (low 32, 0xFFFFFFFF = none), for u32/f32 images.  Word32: 16-bit level and 16-bit
// local parent (0xFFFF = none), for u8/u16 images, whose levels are integers below
// 2^16: half the shared memory per tile, so more tiles are resident per SM.
struct Word64 {
    using T = unsigned long long;
    static constexpr unsigned NO = 0xFFFFFFFFu;
    __device__ static uint32_t key(T w) { return (uint32_t)(w >> 32); }
    __device__ static int par(T w) { return (uint32_t)w == NO ? NONE : (int)(uint32_t)w; }
    __device__ static T make(uint32_t k, int p) { return ((T)k << 32) | (p == NONE ? NO : (uint32_t)p); }
};
struct Word32 {
    using T = unsigned int;
    static constexpr unsigned NO = 0xFFFFu;
    __device__ static uint32_t key(T w) { return w >> 16; }
    __device__ static int par(T w) { return (w & NO) == NO ? NONE : (int)(w & NO); }
    __device__ static T make(uint32_t k, int p) { return (k << 16) | (p == NONE ? NO : (unsigned)p); }
};
template <typename T> struct TileWord { using W = Word64; };
template <> struct TileWord<uint8_t> { using W = Word32; };
template <> struct TileWord<uint16_t> { using W = Word32; };

template <class W>
struct SmemAcc {
    typename W::T *w;
    unsigned *err;
    int npix;
    __device__ typename W::T load(int i) const { return ((volatile typename W::T *)w)[i]; }
    __device__ void store(int i, typename W::T v) { ((volatile typename W::T *)w)[i] = v; }
    __device__ bool cas(int i, typename W::T expect, typename W::T v) { return atomicCAS(w + i, expect, v) == expect; }
    __device__ void error(unsigned bit) { raise_error(err, bit); }
};

// Level root of i (follows equal-key links, path halving); on return i is the root
// and w its word.
template <class W>
__device__ __forceinline__ void levelroot_s(SmemAcc<W> &acc, int &i, typename W::T &w)
{
    w = acc.load(i);
    const uint32_t k = W::key(w);
    for (int it = 0; it <= acc.npix; it++) {
        const int p = W::par(w);
        if (p == NONE) return;
        const typename W::T wp = acc.load(p);
        if (W::key(wp) != k) return;
        const int pp = W::par(wp);
        if (pp != NONE) {
            const typename W::T wpp = acc.load(pp);
            if (W::key(wpp) == k) {
                acc.store(i, W::make(k, pp));
                i = pp;
                w = wpp;
                continue;
            }
        }
        i = p;
        w = wp;
        return;
    }
    acc.error(DEVERR_WALK_BOUND);
}

// connect() on the tile's shared-memory words (the same splices as the HBM
// version, re-reading a parent's word at each step: shared-memory latency is a few
// tens of cycles, and carrying it would cost registers and so occupancy)
template <class W>
__device__ __forceinline__ void connect_s(SmemAcc<W> &acc, int a, int b, long long bound)
{
    typename W::T wa, wb;
    levelroot_s(acc, a, wa);
    levelroot_s(acc, b, wb);
    for (long long it = 0; it < bound; it++) {
        if (a == b) return;
        uint32_t ka = W::key(wa), kb = W::key(wb);
        if (ka < kb || (ka == kb && a < b)) {
            int t = a; a = b; b = t;
            typename W::T tw = wa; wa = wb; wb = tw;
            uint32_t tk = ka; ka = kb; kb = tk;
        }
        const int pa = W::par(wa);
        int lpa = pa;
        typename W::T wl = 0;
        if (pa != NONE) {
            levelroot_s(acc, lpa, wl);
            if (lpa == b) return;
            if (W::key(wl) >= kb) {
                a = lpa;
                wa = wl;
                continue;
            }
        }
        if (acc.cas(a, wa, W::make(ka, b))) {
            if (pa == NONE) return;
            a = b;
            wa = wb;
            b = lpa;
            wb = wl;
        } else {
            levelroot_s(acc, a, wa);
            levelroot_s(acc, b, wb);
        }
    }
    acc.error(DEVERR_MERGE_BOUND);
}

// Max-tree of one tile by the whole CTA.  The tile starts at (x0, y0, z0) of an
// image of geometry g whose pixel (x, y, z) has global index off + z*WH + y*W + x
// (off > 0 for one cutout of a batch).  Writes gval and the tile forest
// (level-root form, global indices, 64-bit order-key words) into gnode.
//
// Shared-memory layout (tile_smem_bytes): the node words alone, with a padded row
// stride RS = tw + 1 (local index of pixel (lx, ly, lz) = lx + ly*RS + lz*RS*th).
// The row pass runs one row per thread in lock-step; unpadded strides would put the
// rows of a warp in one bank.  Nothing else is staged: the row stacks live in the
// parent fields and the level-root form is made in place, so a tile of 4096 u8/u16
// pixels takes 16.5 KB and 12 tiles are resident per SM (8 with a stack array).
template <typename T, bool MIN>
__device__ __forceinline__ void build_tile(const T *__restrict__ img, long long off, const Geom &g, int x0, int y0,
                                           int z0, float gmax, float *__restrict__ gval,
                                           unsigned long long *__restrict__ gnode, unsigned *err, void *smem_raw)
{
    using W = typename TileWord<T>::W;
    using WT = typename W::T;
    constexpr bool NARROW = sizeof(WT) == 4;
    // tile extents from the geometry (at most 4096 pixels: local indices < 2^16)
    const bool is3d = g.D > 1;
    const int TW = g.tw, TH = g.th, TD = g.td;
    const int RS = TW + 1, SLICE = RS * TH, WORDS = RS * TH * TD;
    WT *snode = (WT *)smem_raw;  // WORDS node words
    const int wl = min(TW, g.W - x0), hl = min(TH, g.H - y0), dl = min(TD, g.D - z0);
    const int tid = threadIdx.x, NT = blockDim.x;

    for (int i = tid; i < WORDS; i += NT) {
        int lx = i % RS, ly = (i / RS) % TH, lz = i / SLICE;
        uint32_t k = 0;
        if (lx < wl && ly < hl && lz < dl) {
            long long gp = off + (long long)(z0 + lz) * g.WH + (long long)(y0 + ly) * g.W + (x0 + lx);
            float lv = level_of<T, MIN>(img[gp], gmax);
            gval[gp] = lv;
            k = NARROW ? (uint32_t)lv : order_key(lv);  // u8/u16 levels are integers in [0, 65535]
        }
        snode[i] = W::make(k, NONE);
    }
    __syncthreads();

    // 1-D max-tree of each row with a stack (pop higher keys; the popped chain hangs
    // off the next popped element, the last one off the new pixel).  The stack is a
    // list through the parent fields: a pushed pixel links to the element below it,
    // which is the parent it keeps whether it is popped later (the popped chain) or
    // stays to the end, so popping only re-links the last popped element.
    const int nrows = TH * TD;
    for (int r = tid; r < nrows; r += NT) {
        int ly = r % TH, lz = r / TH;
        if (ly >= hl || lz >= dl) continue;
        const int base = r * RS;
        int top = NONE;
        WT wtop = 0;
        for (int lx = 0; lx < wl; lx++) {
            const int i = base + lx;
            const uint32_t ki = W::key(snode[i]);
            int last = NONE;
            WT wlast = 0;
            while (top != NONE && W::key(wtop) > ki) {
                last = top;
                wlast = wtop;
                top = W::par(wtop);
                if (top != NONE) wtop = snode[top];
            }
            if (last != NONE) snode[last] = W::make(W::key(wlast), i);
            wtop = W::make(ki, top);
            snode[i] = wtop;
            top = i;
        }
    }
    __syncthreads();

    SmemAcc<W> acc{snode, err, WORDS};
    const long long bound = merge_bound_smem(g);
    // merge row bands along y (each z slice), then slabs along z; at level k the
    // seams are the rows (slices) c with c % 2^(k+1) == 2^k.  All edges across the
    // seams of a level at once; correctness does not depend on the order (see
    // connect).  Levels are ordered for shorter merge walks, not for correctness:
    // without the barrier warps run ahead into the next level.
    if (!is3d) {
        // 2-D (4- or 8-connectivity): pixel p on seam row ly joins q0 above it and,
        // with 8-connectivity, the diagonals q0 - 1 and q0 + 1 unless implied: a
        // diagonal p-qd is left out when p's row neighbour toward qd or q0 has a key
        // >= min(key p, key qd), the rule edge_implied states.  Keys never change, so
        // each is read once.  Thread t starts at item t (x = t % TW, seam t / TW) and
        // steps NT items with a carry instead of dividing.
        const bool diag = g.conn == 8;
        const int stepx = NT % TW, stepl = NT / TW;
        for (int half = 1; half < TH; half <<= 1) {
            const int nseams = (TH + 2 * half - 1) / (2 * half);
            for (int lx = tid % TW, s = tid / TW; s < nseams;) {
                const int ly = s * 2 * half + half;
                if (lx < wl && ly < hl) {
                    const int p = lx + ly * RS, q0 = p - RS;
                    connect_s(acc, p, q0, bound);
                    if (diag) {
                        const uint32_t kp = W::key(acc.load(p)), k0 = W::key(acc.load(q0));
                        if (lx > 0) {
                            const uint32_t kd = W::key(acc.load(q0 - 1)), m = kp < kd ? kp : kd;
                            if (k0 < m && W::key(acc.load(p - 1)) < m) connect_s(acc, p, q0 - 1, bound);
                        }
                        if (lx + 1 < wl) {
                            const uint32_t kd = W::key(acc.load(q0 + 1)), m = kp < kd ? kp : kd;
                            if (k0 < m && W::key(acc.load(p + 1)) < m) connect_s(acc, p, q0 + 1, bound);
                        }
                    }
                }
                lx += stepx;
                s += stepl;
                if (lx >= TW) {
                    lx -= TW;
                    s++;
                }
            }
            if (g.level_sync) __syncthreads();
        }
    }
    const Offs offs = forward_offsets(g.conn);
    for (int axis = 1; is3d && axis <= 2; axis++) {
        const int ext = axis == 1 ? TH : TD;
        for (int half = 1; half < ext; half <<= 1) {
            const int nseams = (ext + 2 * half - 1) / (2 * half);
            const int other = axis == 1 ? TD : TH;  // slices (axis y) or rows (axis z)
            const int work = nseams * other * TW;  // at most 4096 * 26
            for (int w = tid; w < work; w += NT) {
                int lx = w % TW;
                int rest = w / TW;
                int o = rest % other;
                int s = rest / other;
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
                    const int qi = qx + qy * RS + qz * SLICE;
                    if (offs.n > 3) {  // 8/26-connectivity: skip diagonal edges implied by others
                        const uint32_t kp = W::key(acc.load(p)), kq = W::key(acc.load(qi));
                        auto key_at = [&](int sx, int sy, int sz) {
                            return W::key(acc.load(p + sx + sy * RS + sz * SLICE));
                        };
                        if (edge_implied(-dx, -dy, -dz, kp < kq ? kp : kq, key_at)) continue;
                    }
                    connect_s(acc, p, qi, bound);
                }
            }
            if (g.level_sync) __syncthreads();
        }
    }
    __syncthreads();

    // level-root form inside the tile: pixel -> level root, root -> parent's level
    // root; to global indices.  A flat zone of F pixels can be a chain of ~F
    // equal-key links, so walking it from every pixel would cost O(F^2): instead
    // every pixel whose parent is not its level root jumps to its grandparent, in
    // place, round by round.  A word read while its owner rewrites it is the old or
    // the new link, both equal-key ancestors, so each round at least halves every
    // distance to a level root as synchronous doubling does: at most
    // log2(WORDS) + 1 rounds change anything.
    for (int round = 0;; round++) {
        int moved = 0;
        for (int i = tid; i < WORDS; i += NT) {
            const WT w = acc.load(i);  // padding and outside pixels: no parent
            const int p = W::par(w);
            if (p == NONE) continue;
            const WT wp = acc.load(p);
            if (W::key(wp) != W::key(w)) continue;  // a level root
            const int pp = W::par(wp);
            if (pp == NONE || W::key(acc.load(pp)) != W::key(w)) continue;  // p is the level root
            acc.store(i, W::make(W::key(w), pp));
            moved = 1;
        }
        if (!__syncthreads_or(moved)) break;
        if (round > 16) {
            acc.error(DEVERR_WALK_BOUND);
            break;
        }
    }
    for (int i = tid; i < WORDS; i += NT) {
        int lx = i % RS, ly = (i / RS) % TH, lz = i / SLICE;
        if (lx >= wl || ly >= hl || lz >= dl) continue;
        const WT w = snode[i];
        int p = W::par(w);
        if (p != NONE) {
            const WT wp = snode[p];
            if (W::key(wp) != W::key(w)) {  // i is a level root: its parent node's level root
                const int pp = W::par(wp);
                if (pp != NONE && W::key(snode[pp]) == W::key(wp)) p = pp;
            }
        }
        int out = NONE;
        if (p != NONE) {
            int px = p % RS, py = (p / RS) % TH, pz = p / SLICE;
            out = (int)(off + (long long)(z0 + pz) * g.WH + (long long)(y0 + py) * g.W + (x0 + px));
        }
        long long gp = off + (long long)(z0 + lz) * g.WH + (long long)(y0 + ly) * g.W + (x0 + lx);
        const uint32_t key = NARROW ? order_key((float)W::key(w)) : W::key(w);
        gnode[gp] = wmake(key, out);
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
