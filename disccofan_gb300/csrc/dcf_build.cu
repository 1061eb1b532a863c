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
void launch_canon(unsigned long long *node, const Geom &g, int *parent, unsigned char *isroot,
                  unsigned long long *num_nodes, unsigned *err, int sm_count, cudaStream_t s)
{
    prof_begin(P_CANON, s);
    k_canon<<<grid_for(g.N, 256, sm_count), 256, 0, s>>>(node, g, parent, isroot, num_nodes, err);
    prof_end(P_CANON, s);
}

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
    launch_canon(a.node, a.g, a.parent, a.isroot, a.num_nodes, a.err, a.sm_count, s);
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
