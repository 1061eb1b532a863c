// Internal device/host definitions shared by the CUDA translation units.
//
// Data layout in HBM (one tree):
//   img      caller's pixels in their own type (u8/u16/u32/f32), x fastest; read
//            once by the tile kernel.
//   gval     float[N]: the grey levels (min-tree: inverted) every later pass uses.
//   node     uint64[N] (build scratch): key and current parent of every pixel
//            while trees are merged; see wmake/wkey/wpar.
//   parent   int32[N]: canonical form after the build -- a pixel that is not a
//            level root points to its node's level root (the lowest linear index
//            of the node's flat zone, the reference's choice, flood.c:127-141); a
//            level root points to its parent node's level root; the root holds -1.
//   attribute records: structure-of-arrays indexed by pixel, valid at level roots.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "dcf_eigen.h"

namespace dcf {

constexpr int NONE = -1;

enum DType : int { U8 = 0, U16 = 1, U32 = 2, F32 = 3 };

// Error bits raised by kernels into a device word the host checks.
enum DevErr : unsigned {
    DEVERR_MERGE_BOUND = 1u << 0,   // a merge loop exceeded its iteration bound
    DEVERR_WALK_BOUND = 1u << 1,    // a tree walk exceeded its iteration bound
    DEVERR_WAIT_BOUND = 1u << 2,    // a bounded wait gave up (work queue / flag)
    DEVERR_CAPACITY = 1u << 3,      // a fixed-capacity work list overflowed (results incomplete)
};

struct Geom {
    int W, H, D;
    long long WH;
    long long N;
    int conn;
    int tw, th, td;  // build tile extents (tw*th*td <= 4096)
    int level_sync;  // barrier between the band-merge levels of a tile
    long long merge_bound;  // iteration limit of the merge loops (0: the built-in limits)
};

// Grey level as the reference holds it (types.h:53 `value` = float): the pixel
// converted to float, inverted as max - v for a min-tree (preprocessing.c:84-91).
template <typename T>
__device__ __forceinline__ float to_float(T v);
template <> __device__ __forceinline__ float to_float<uint8_t>(uint8_t v) { return (float)v; }
template <> __device__ __forceinline__ float to_float<uint16_t>(uint16_t v) { return (float)v; }
template <> __device__ __forceinline__ float to_float<uint32_t>(uint32_t v) { return __uint2float_rn(v); }
template <> __device__ __forceinline__ float to_float<float>(float v) { return v; }

template <typename T, bool MIN>
__device__ __forceinline__ float level_of(T raw, float gmax)
{
    float v = to_float<T>(raw);
    return MIN ? __fsub_rn(gmax, v) : v;
}

// Order-preserving unsigned key of a float level (the reference's transform_float,
// flood.c:362-371).  -0.0 is folded onto +0.0 first because the reference treats
// them as one grey level (its flat-zone test is float ==).
__device__ __forceinline__ uint32_t order_key(float v)
{
    uint32_t u = __float_as_uint(v);
    if (u == 0x80000000u) u = 0u;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_to_level(uint32_t k)
{
    uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    return __uint_as_float(u);
}

// Forward half-neighbourhoods (offsets with a larger linear index) per connectivity.
// 2-D 4: +x, +y.  2-D 8: +x, +y, (+1,+1), (-1,+1).  3-D 6: +x, +y, +z.
// 3-D 26: the 13 offsets (dx,dy,dz) lexicographically after (0,0,0).
struct Offs {
    int n;
    signed char d[13][3];
};

__host__ __device__ inline Offs forward_offsets(int conn)
{
    Offs o{};
    auto add = [&](int dx, int dy, int dz) {
        o.d[o.n][0] = (signed char)dx;
        o.d[o.n][1] = (signed char)dy;
        o.d[o.n][2] = (signed char)dz;
        o.n++;
    };
    if (conn == 4 || conn == 6 || conn == 8) {
        add(1, 0, 0);
        add(0, 1, 0);
        if (conn == 6) add(0, 0, 1);
        if (conn == 8) {
            add(1, 1, 0);
            add(-1, 1, 0);
        }
    } else {  // 26
        for (int dz = 0; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (dz == 0 && (dy < 0 || (dy == 0 && dx <= 0))) continue;
                    add(dx, dy, dz);
                }
    }
    return o;
}

// Edges implied by others.  An edge from p to q = p + (ex, ey, ez) with two or three
// non-zero components can be left out when some pixel r = p + s, s a proper part of
// the offset (some of its non-zero components, not all), has level >= min(level p,
// level q): the path p - r - q is made of two edges with fewer non-zero components
// and joins p and q at every threshold at or below the edge's level, so the max-tree
// is the same without the edge.  Straight edges are never left out, so by induction
// over the number of non-zero components every dropped edge is implied by kept ones,
// whichever phase (row pass, band merge, seam merge) handles those.  The 8- and
// 26-neighbourhoods hold every part of each of their offsets.  key_at(sx, sy, sz)
// returns the order key of pixel p + (sx, sy, sz).
template <class KeyAt>
__device__ __forceinline__ bool edge_implied(int ex, int ey, int ez, uint32_t kmin, KeyAt key_at)
{
    const int nz = (ex != 0) | ((ey != 0) << 1) | ((ez != 0) << 2);
    if (__popc(nz) < 2) return false;
    for (int m = 1; m < 7; m++) {
        if ((m & ~nz) || m == nz) continue;
        if (key_at(m & 1 ? ex : 0, m & 2 ? ey : 0, m & 4 ? ez : 0) >= kmin) return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// Lock-free concurrent merge of two branches of a max-tree forest.
//
// Invariant kept by every writer: par[x] is NONE, or key(par[x]) <= key(x), and
// a link between equal keys goes to a LOWER index.  A pixel x is a level root iff
// par[x] == NONE or key(par[x]) < key(x); following equal-key links from any
// pixel ends at the lowest index of its flat zone.
//
// connect(a, b) makes the root paths of a and b one sorted chain (the merge of
// Wilkinson et al.'s concurrent filter, the reference's merge_nodes flood.c:292-353),
// but without locks: the only write that changes structure is a CAS that splices
// node b between a and a's parent pa (key(pa) < key(b) <= key(a)); the displaced
// tail pa is then merged into b's chain by the same thread.  Every successful CAS
// raises par[a]'s key, so the loop terminates; links are only ever created between
// pixels connected at or above the lower key, so at quiescence the forest is the
// component tree of all merged edges.  Path halving writes only shortcut
// equal-key links, which no CAS can race with (a CAS expects a lower-key parent).
// ---------------------------------------------------------------------------
// Node words: one 64-bit word per pixel holds its immutable key (high half) and
// its current parent (low half, 0xFFFFFFFF = none), so one dependent load yields
// both the next node on a chain and the key needed to compare it, and a splice is a
// single 64-bit CAS.
__device__ __forceinline__ int wpar(uint64_t w)
{
    uint32_t p = (uint32_t)w;
    return p == 0xFFFFFFFFu ? NONE : (int)p;
}
__device__ __forceinline__ uint32_t wkey(uint64_t w) { return (uint32_t)(w >> 32); }
__device__ __forceinline__ uint64_t wmake(uint32_t key, int par)
{
    return ((uint64_t)key << 32) | (uint32_t)(par == NONE ? 0xFFFFFFFFu : (uint32_t)par);
}

// Level root of i given its word w, continuing past equal-key links (with path
// halving); on return (i, w) is the level root and (ni, nw) the first pixel of
// the parent node and its word (ni = NONE at a root).  The parent's word is the
// one this walk had to load anyway to see the key change, so a caller stepping
// down a chain pays one dependent load per node.
template <class A>
__device__ __forceinline__ void levelroot_next(A &acc, int &i, uint64_t &w, int &ni, uint64_t &nw)
{
    const uint32_t k = wkey(w);
    const long long bound = acc.walk_bound();
    for (long long it = 0; it < bound; it++) {
        const int p = wpar(w);
        if (p == NONE) {
            ni = NONE;
            return;
        }
        const uint64_t wp = acc.load(p);
        if (wkey(wp) != k) {
            ni = p;
            nw = wp;
            return;
        }
        const int pp = wpar(wp);
        if (pp == NONE) {
            i = p;
            w = wp;
            ni = NONE;
            return;
        }
        const uint64_t wpp = acc.load(pp);
        if (wkey(wpp) == k) {
            acc.store(i, wmake(k, pp));
            i = pp;
            w = wpp;
            continue;
        }
        i = p;
        w = wp;
        ni = pp;
        nw = wpp;
        return;
    }
    ni = NONE;
    acc.error(DEVERR_WALK_BOUND);
}

// Every (x, wx) pair below is read in the order word of x, then word of its parent
// (nx, nwx); a pair may be older than other threads' writes, like the view of a
// delayed thread, and structure only changes through a CAS on the exact word held.
template <class A>
__device__ __forceinline__ void connect(A &acc, int a, int b, long long bound)
{
    uint64_t wa = acc.load(a), wb = acc.load(b), nwa = 0, nwb = 0;
    int na, nb;
    levelroot_next(acc, a, wa, na, nwa);
    levelroot_next(acc, b, wb, nb, nwb);
    for (long long it = 0; it < bound; it++) {
        if (a == b) return;
        uint32_t ka = wkey(wa), kb = wkey(wb);
        if (ka < kb || (ka == kb && a < b)) {
            int t = a; a = b; b = t;
            uint64_t tw = wa; wa = wb; wb = tw;
            t = na; na = nb; nb = t;
            tw = nwa; nwa = nwb; nwb = tw;
            uint32_t tk = ka; ka = kb; kb = tk;
        }
        // a sits above b: ka > kb, or equal keys with a > b (a's node joins b's)
        int lpa = na, nl = NONE;
        uint64_t wl = nwa, nwl = 0;
        if (na != NONE) {
            levelroot_next(acc, lpa, wl, nl, nwl);
            if (lpa == b) return;
            if (wkey(wl) >= kb) {  // b belongs below a's parent node: descend
                a = lpa;
                wa = wl;
                na = nl;
                nwa = nwl;
                continue;
            }
        }
        if (acc.cas(a, wa, wmake(ka, b))) {
            if (na == NONE) return;
            // merge the displaced tail (a's old parent node) into b's chain
            a = b;
            wa = wb;
            na = nb;
            nwa = nwb;
            b = lpa;
            wb = wl;
            nb = nl;
            nwb = nwl;
        } else {
            wa = acc.load(a);
            levelroot_next(acc, a, wa, na, nwa);
            wb = acc.load(b);
            levelroot_next(acc, b, wb, nb, nwb);
        }
    }
    acc.error(DEVERR_MERGE_BOUND);
}

__device__ __forceinline__ void raise_error(unsigned *err, unsigned bit)
{
    if (err) atomicOr(err, bit);
}

}  // namespace dcf
