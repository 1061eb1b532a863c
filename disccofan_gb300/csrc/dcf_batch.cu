// Batched max-trees of many 2-D cutouts of different sizes (no reference
// counterpart: the reference processes one image per run).
//
// All cutouts' pixels are concatenated; cutout i occupies indices [off_i, off_i +
// W_i*H_i).  The work is described by a tile list: every cutout is cut into tiles
// of the batch's tile shape, and each tile descriptor names its cutout.  Trees of
// different cutouts never touch, so after the per-tile build and the seam merge
// (both restricted to one cutout) every remaining pass -- canonical form,
// bottom-up attributes, pointer jumping, filtering -- runs unchanged on the
// concatenation.
//
//   k_batch_tile_build   persistent: grid = SMs x CTAs-per-SM; each CTA takes the
//                        next tiles from an atomic work counter until none is left.
//   k_batch_seam(_collect)  tile-boundary edges inside each cutout, merged at once
//                        or collected for the level-ordered merge.
//   k_batch_attr_pixels  per-pixel attribute contributions, walked tile by tile so
//                        each pixel's cutout (and in-cutout coordinates) is known.
//   k_batch_spectrum     per-cutout 2-D pattern spectra, one shared-memory
//                        histogram per tile.
#include "dcf_tile.cuh"
#include "dcf_attr_eval.cuh"

namespace dcf {

static __device__ __forceinline__ Geom cut_geom(const BatchImg &im, const Geom &bg)
{
    Geom g = bg;
    g.W = im.W;
    g.H = im.H;
    g.D = 1;
    g.WH = (long long)im.W * im.H;
    g.N = g.WH;
    return g;
}

// Persistent work queue: each CTA grabs `chunk` consecutive tiles at a time from
// the atomic counter *next until the list is exhausted.  Every grab advances the
// counter, so the loop ends after at most ntiles / chunk + 1 grabs per CTA.
template <typename T>
__global__ void __launch_bounds__(TileCfg<T>::threads, TileCfg<T>::min_blocks)
k_batch_tile_build(const T *__restrict__ img, Geom bg, const BatchImg *__restrict__ imgs,
                   const BatchTile *__restrict__ tiles, int ntiles, int chunk, unsigned *next,
                   float *__restrict__ gval, unsigned long long *__restrict__ gnode, unsigned *err)
{
    extern __shared__ unsigned long long smem_tile[];
    __shared__ int s_first;
    for (int grab = 0; grab <= ntiles / chunk + 1; grab++) {
        if (threadIdx.x == 0) s_first = (int)atomicAdd(next, (unsigned)chunk);
        __syncthreads();
        const int first = s_first;
        if (first >= ntiles) break;
        for (int t = first; t < min(first + chunk, ntiles); t++) {
            const BatchTile tl = tiles[t];
            const BatchImg im = imgs[tl.img];
            const Geom g = cut_geom(im, bg);
            build_tile<T, false>(img, im.off, g, tl.x0, tl.y0, 0, 0.0f, gval, gnode, err, smem_tile);
            __syncthreads();  // the shared buffers (and s_first) are reused next
        }
    }
}

// the largest shared-memory split of the SM for the tile kernels (once per process)
static void batch_tile_carveout()
{
    static bool done = (cudaFuncSetAttribute(k_batch_tile_build<uint8_t>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared),
                        cudaFuncSetAttribute(k_batch_tile_build<uint16_t>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared),
                        cudaFuncSetAttribute(k_batch_tile_build<uint32_t>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared),
                        cudaFuncSetAttribute(k_batch_tile_build<float>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared),
                        true);
    (void)done;
}

// Seam edges of a batch: work item = (tile, face, face pixel, forward offset) over
// the tile's +x, -x and +y faces; face f takes the offsets pointing out through
// it.  2-D forward offsets never point to -y, so every edge between two tiles of
// one cutout leaves its low endpoint's tile through one of these faces.  Edges
// leaving the cutout are skipped, and so are diagonal edges implied by others
// (edge_implied).  One connect per edge and thread.
__device__ __forceinline__ bool batch_seam_item(const Geom &bg, const BatchImg *imgs, const BatchTile *tiles,
                                                const Offs &offs, int fmax, long long w,
                                                const unsigned long long *gnode, int &p, int &q)
{
    const int e = (int)(w % offs.n);
    long long r = w / offs.n;
    const int k = (int)(r % fmax);
    r /= fmax;
    const int f = (int)(r % 3);
    const int t = (int)(r / 3);
    const int dx = offs.d[e][0], dy = offs.d[e][1];
    if (!(f == 0 ? dx > 0 : f == 1 ? dx < 0 : dy > 0)) return false;
    const BatchTile tl = tiles[t];
    const BatchImg im = imgs[tl.img];
    const int wl = min(bg.tw, im.W - tl.x0), hl = min(bg.th, im.H - tl.y0);
    if (k >= (f <= 1 ? hl : wl)) return false;
    const int x = tl.x0 + (f == 0 ? wl - 1 : (f == 1 ? 0 : k));
    const int y = tl.y0 + (f <= 1 ? k : hl - 1);
    const int qx = x + dx, qy = y + dy;
    if (qx < 0 || qx >= im.W || qy >= im.H) return false;
    p = (int)(im.off + (long long)y * im.W + x);
    q = (int)(im.off + (long long)qy * im.W + qx);
    if (offs.n > 3) {
        const unsigned kp = wkey(gnode[p]), kq = wkey(gnode[q]);
        const int pp = p, W = im.W;
        auto key_at = [&](int sx, int sy, int) { return wkey(gnode[pp + (long long)sy * W + sx]); };
        if (edge_implied(dx, dy, 0, kp < kq ? kp : kq, key_at)) return false;
    }
    return true;
}

__global__ void k_batch_seam(unsigned long long *gnode, Geom bg, const BatchImg *__restrict__ imgs,
                             const BatchTile *__restrict__ tiles, int ntiles, unsigned *err)
{
    GlobalAcc acc{gnode, err, bg.N};
    const Offs offs = forward_offsets(bg.conn);
    const int fmax = bg.tw > bg.th ? bg.tw : bg.th;
    const long long work = (long long)ntiles * 3 * fmax * offs.n;
    for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < work;
         w += (long long)gridDim.x * blockDim.x) {
        int p, q;
        if (batch_seam_item(bg, imgs, tiles, offs, fmax, w, gnode, p, q)) connect(acc, p, q, merge_bound_global(bg));
    }
}

__global__ void k_batch_seam_collect(const unsigned long long *gnode, Geom bg, const BatchImg *__restrict__ imgs,
                                     const BatchTile *__restrict__ tiles, int ntiles, SeamEdges e)
{
    const Offs offs = forward_offsets(bg.conn);
    const int fmax = bg.tw > bg.th ? bg.tw : bg.th;
    const long long work = (long long)ntiles * 3 * fmax * offs.n;
    const int lane = threadIdx.x & 31;
    for (long long base = blockIdx.x * (long long)blockDim.x + threadIdx.x - lane; base < work;
         base += (long long)gridDim.x * blockDim.x) {
        int p = 0, q = 0;
        const bool valid = base + lane < work && batch_seam_item(bg, imgs, tiles, offs, fmax, base + lane, gnode, p, q);
        seam_append(e, gnode, valid, p, q);
    }
}

long long batch_seam_edge_bound(const Geom &bg, const BatchImg *imgs, int count)
{
    const Offs o = forward_offsets(bg.conn);
    int npx = 0, nmx = 0, npy = 0;
    for (int i = 0; i < o.n; i++) {
        npx += o.d[i][0] > 0;
        nmx += o.d[i][0] < 0;
        npy += o.d[i][1] > 0;
    }
    long long b = 0;
    for (int i = 0; i < count; i++) {
        const long long ntx = (imgs[i].W + bg.tw - 1) / bg.tw, nty = (imgs[i].H + bg.th - 1) / bg.th;
        b += ntx * nty * ((long long)bg.th * (npx + nmx) + (long long)bg.tw * npy);
    }
    return b;
}

// Per-pixel contributions, tile by tile (x, y are coordinates inside the cutout,
// as the reference would see the cutout on its own).  Area is aggregated over the
// lanes of a warp that share a node, the bounding box likewise.
template <int G, bool EXACT>
__global__ void k_batch_attr_pixels(const float *__restrict__ gval, Geom bg, const BatchImg *__restrict__ imgs,
                                    const BatchTile *__restrict__ tiles, int ntiles, const int *__restrict__ parent,
                                    const unsigned char *__restrict__ isroot, AttrBufs a)
{
    const int lane = threadIdx.x & 31;
    const int TW = bg.tw, TP = bg.tw * bg.th;
    const long long work = (long long)ntiles * TP;
    const long long wstride = (long long)gridDim.x * blockDim.x;
    // warp-uniform loop: every lane runs the same iterations (the match/reduce
    // intrinsics below need the whole warp)
    for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane; base < work; base += wstride) {
        const long long w = base + lane;
        bool valid = w < work;
        long long p = 0;
        unsigned x = 0, y = 0;
        if (valid) {
            const BatchTile tl = tiles[w / TP];
            const BatchImg im = imgs[tl.img];
            const int li = (int)(w % TP), lx = li % TW, ly = li / TW;
            valid = tl.x0 + lx < im.W && tl.y0 + ly < im.H;
            x = tl.x0 + lx;
            y = tl.y0 + ly;
            p = im.off + (long long)y * im.W + x;
        }
        const int par = valid ? parent[p] : NONE;
        const bool root = valid && isroot[p];
        const int node = valid ? (root ? (int)p : par) : -2;
        if (root && par != NONE) atomicAdd(a.pending + par, 1);
        const unsigned grp = __match_any_sync(0xffffffffu, node);
        const bool leader = lane == __ffs(grp) - 1;
        if (valid && leader) atomicAdd(a.area + node, (unsigned)__popc(grp));
        if (G == 0 || !valid) continue;
        if (G == 1) {
            const unsigned mnx = __reduce_min_sync(grp, x), mny = __reduce_min_sync(grp, y);
            const unsigned mxx = __reduce_max_sync(grp, x + 1), mxy = __reduce_max_sync(grp, y + 1);
            if (leader) {
                atomicMin(a.bmin[0] + node, mnx);
                atomicMin(a.bmin[1] + node, mny);
                atomicMax(a.bmax[0] + node, mxx);
                atomicMax(a.bmax[1] + node, mxy);
            }
            continue;
        }
        if (G == 2 || G == 4) {
            atomicAdd(a.s1[0] + node, (unsigned long long)x);
            atomicAdd(a.s1[1] + node, (unsigned long long)y);
        }
        if (G == 4) {
            atomicAdd(a.s2[0] + node, (unsigned long long)x * x);
            atomicAdd(a.s2[1] + node, (unsigned long long)y * y);
            atomicAdd(a.s2[3] + node, (unsigned long long)x * y);
        }
        if (G == 3 || (G == 4 && a.grey)) {
            const float gv = gval[p];
            if (EXACT) {
                const long long gi = (long long)gv;
                atomicAdd((unsigned long long *)a.gw[0] + node, (unsigned long long)gi);
                atomicAdd((unsigned long long *)a.gw[2] + node, (unsigned long long)(gi * (long long)x));
                atomicAdd((unsigned long long *)a.gw[3] + node, (unsigned long long)(gi * (long long)y));
            } else {
                const double gd = (double)gv;
                atomicAdd((double *)a.gw[0] + node, gd);
                atomicAdd((double *)a.gw[2] + node, gd * (double)x);
                atomicAdd((double *)a.gw[3] + node, gd * (double)y);
            }
        }
    }
}

// find_scale (pattern.c:7-24): the last bin whose lambda is <= the attribute
__device__ __forceinline__ int find_scale_b(const float *lv, int n, double v)
{
    int upper = n - 1, lower = 0;
    if (v >= (double)lv[upper]) return upper;
    int mid = (upper + lower) / 2;
    while (mid != lower) {
        if (v >= (double)lv[mid]) lower = mid;
        else upper = mid;
        mid = (upper + lower) / 2;
    }
    return lower;
}

// Per-cutout 2-D pattern spectra: spec[img * n1 * n2 + s1 + s2 * n1] += dh * area
// over the level roots of the cutout (dh in float, as pattern.c:175-186).  A block
// takes whole tiles (each inside one cutout), accumulates a tile in a shared-memory
// histogram and flushes its non-zero bins with global atomics; with more than
// SPEC_BATCH_SMEM_BINS bins it adds to global memory directly.
constexpr int SPEC_BATCH_SMEM_BINS = 4096;

template <bool SMEM>
__global__ void k_batch_spectrum(Geom bg, const BatchImg *__restrict__ imgs, const BatchTile *__restrict__ tiles,
                                 int ntiles, const int *__restrict__ parent, const unsigned char *__restrict__ isroot,
                                 const float *__restrict__ gval, AttrBufs a, int a1, const float *__restrict__ l1,
                                 int n1, int a2, const float *__restrict__ l2, int n2, float pd0, float pd1, float pd2,
                                 double *spec)
{
    __shared__ double hist[SMEM ? SPEC_BATCH_SMEM_BINS : 1];
    const float pd[3] = {pd0, pd1, pd2};
    const int TW = bg.tw, TP = bg.tw * bg.th, nb = n1 * n2;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BatchTile tl = tiles[t];
        const BatchImg im = imgs[tl.img];
        double *dst = spec + (long long)tl.img * nb;
        if (SMEM) {
            for (int i = threadIdx.x; i < nb; i += blockDim.x) hist[i] = 0.0;
            __syncthreads();
        }
        for (int li = threadIdx.x; li < TP; li += blockDim.x) {
            const int lx = li % TW, ly = li / TW;
            if (tl.x0 + lx >= im.W || tl.y0 + ly >= im.H) continue;
            const long long p = im.off + (long long)(tl.y0 + ly) * im.W + (tl.x0 + lx);
            if (!isroot[p]) continue;
            const int q = parent[p];
            const float dh = q != NONE ? __fsub_rn(gval[p], gval[q]) : gval[p];
            if (dh == 0.0f) continue;
            const double ar = area_value(a, (int)p, pd);
            const int s1 = find_scale_b(l1, n1, a1 < 0 ? ar : attr_value(a, a1, (int)p, pd));
            const int s2 = n2 <= 1 ? 0 : find_scale_b(l2, n2, a2 < 0 ? ar : attr_value(a, a2, (int)p, pd));
            if (SMEM) atomicAdd(hist + s1 + s2 * n1, (double)dh * ar);
            else atomicAdd(dst + s1 + s2 * n1, (double)dh * ar);
        }
        if (SMEM) {
            __syncthreads();
            for (int i = threadIdx.x; i < nb; i += blockDim.x)
                if (hist[i] != 0.0) atomicAdd(dst + i, hist[i]);
            __syncthreads();
        }
    }
}

void launch_batch_build(int dtype, const void *img, const Geom &bg, const BatchImg *imgs, const BatchTile *tiles,
                        int ntiles, int chunk, unsigned *next, float *gval, unsigned long long *node, int *parent,
                        unsigned char *isroot, unsigned long long *num_nodes, int *nodes, unsigned *err,
                        int ctas_per_sm, SeamEdges &seam, int sm, cudaStream_t s)
{
    const int grid = sm * ctas_per_sm;
    batch_tile_carveout();
    cudaMemsetAsync(next, 0, sizeof(unsigned), s);
    prof_begin(P_TILE, s);
#define DCF_TB(T)                                                                                       \
    k_batch_tile_build<T><<<grid, TileCfg<T>::threads, tile_smem_bytes(bg.tw, bg.th, 1, TileCfg<T>::word_bytes), s>>>((const T *)img, bg, imgs, tiles, ntiles, chunk, \
                                                          next, gval, node, err); note_launch()
    switch (dtype) {
    case U8: DCF_TB(uint8_t); break;
    case U16: DCF_TB(uint16_t); break;
    case U32: DCF_TB(uint32_t); break;
    default: DCF_TB(float); break;
    }
#undef DCF_TB
    prof_end(P_TILE, s);
    prof_begin(P_SEAM, s);
    const int fmax = bg.tw > bg.th ? bg.tw : bg.th;
    const long long work = (long long)ntiles * 3 * fmax * forward_offsets(bg.conn).n;
    if (seam.buckets > 0) {
        cudaMemsetAsync(seam.count, 0, 4, s);
        cudaMemsetAsync(seam.hist, 0, 4 * SEAM_BINS, s);
        k_batch_seam_collect<<<grid_for(work, 256, sm), 256, 0, s>>>(node, bg, imgs, tiles, ntiles, seam); note_launch();
        launch_seam_buckets(seam, node, bg.N, bg.merge_bound, err, sm, s);
    } else {
        k_batch_seam<<<grid_for(work, 128, sm), 128, 0, s>>>(node, bg, imgs, tiles, ntiles, err); note_launch();
    }
    prof_end(P_SEAM, s);
    launch_canon(node, bg, parent, isroot, num_nodes, nodes, err, sm, s);
}

void launch_batch_attr_pixels(const Geom &bg, const BatchImg *imgs, const BatchTile *tiles, int ntiles,
                              const float *gval, const int *parent, const unsigned char *isroot, AttrBufs &a, int sm,
                              cudaStream_t s)
{
    const long long work = (long long)ntiles * bg.tw * bg.th;
    const int nb = grid_for(work, 256, sm);
    prof_begin(P_ATTR_PIX, s);
#define DCF_BP(G, E) k_batch_attr_pixels<G, E><<<nb, 256, 0, s>>>(gval, bg, imgs, tiles, ntiles, parent, isroot, a); note_launch()
    switch (a.group * 2 + (a.exact_g ? 1 : 0)) {
    case 0: case 1: DCF_BP(0, false); break;
    case 2: case 3: DCF_BP(1, false); break;
    case 4: case 5: DCF_BP(2, false); break;
    case 6: DCF_BP(3, false); break;
    case 7: DCF_BP(3, true); break;
    case 8: DCF_BP(4, false); break;
    default: DCF_BP(4, true); break;
    }
#undef DCF_BP
    prof_end(P_ATTR_PIX, s);
}

void launch_batch_spectrum(const Geom &bg, const BatchImg *imgs, const BatchTile *tiles, int ntiles, const int *parent,
                           const unsigned char *isroot, const float *gval, const AttrBufs &a, int a1, const float *l1,
                           int n1, int a2, const float *l2, int n2, const float *pixdim, double *spec, int sm,
                           cudaStream_t s)
{
    const int grid = ntiles < sm * 8 ? ntiles : sm * 8;
    prof_begin(P_SPECTRUM, s);
    if ((long long)n1 * n2 <= SPEC_BATCH_SMEM_BINS)
        k_batch_spectrum<true><<<grid, 256, 0, s>>>(bg, imgs, tiles, ntiles, parent, isroot, gval, a, a1, l1, n1, a2,
                                                    l2, n2, pixdim[0], pixdim[1], pixdim[2], spec);
    else
        k_batch_spectrum<false><<<grid, 256, 0, s>>>(bg, imgs, tiles, ntiles, parent, isroot, gval, a, a1, l1, n1, a2,
                                                     l2, n2, pixdim[0], pixdim[1], pixdim[2], spec);
    note_launch();
    prof_end(P_SPECTRUM, s);
}

}  // namespace dcf

namespace dcf {

// CTAs of the persistent tile kernel that fit on one SM for a tile shape (with the
// largest shared-memory split, which launch_batch_build asks for too)
int batch_max_ctas_per_sm(int dtype, int tw, int th)
{
    batch_tile_carveout();
    int n = 0;
#define DCF_OCC(T)                                                                                       \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_tile_build<T>, TileCfg<T>::threads,      \
                                                  tile_smem_bytes(tw, th, 1, TileCfg<T>::word_bytes))
    switch (dtype) {
    case U8: DCF_OCC(uint8_t); break;
    case U16: DCF_OCC(uint16_t); break;
    case U32: DCF_OCC(uint32_t); break;
    default: DCF_OCC(float); break;
    }
#undef DCF_OCC
    return n;
}

}  // namespace dcf
