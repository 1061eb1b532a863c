// Attribute accumulation and readout (the reference's attribute vtable,
// attributes.c:47-880 + 1201-1248, and its merges during flooding, flood.c:239-240,
// re-designed as two passes over the finished tree):
//
//   k_attr_pixels  every pixel adds its own contribution (area, bounding box,
//                  coordinate and grey-weighted moments) to its node's record;
//                  area updates are warp-aggregated (lanes of one flat zone add once).
//                  Level roots count their children in `pending`.
//   k_mark_leaves  nodes without children are tagged (pending = -1).
//   k_attr_up      bottom-up fold: a thread starts at every leaf, adds its record
//                  into the parent, and only the thread that brings a parent's
//                  pending count to zero continues upward with the completed record.
//
// Coordinate moments are summed as exact 64-bit integers (the reference sums them in
// double, which is exact below 2^53); grey-weighted moments are exact 64-bit integers
// for 8/16-bit images and doubles otherwise.  Readouts (k_node_attr and the device
// function attr_value) follow the reference's expressions operand by operand,
// including which factors are float and which double.
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
        const unsigned x = (unsigned)(p % g.W), y = (unsigned)((p / g.W) % g.H), z = (unsigned)(p / g.WH);
        if (G == 1) {
            atomicMin(a.bmin[0] + node, x);
            atomicMin(a.bmin[1] + node, y);
            atomicMin(a.bmin[2] + node, z);
            atomicMax(a.bmax[0] + node, x + 1);
            atomicMax(a.bmax[1] + node, y + 1);
            atomicMax(a.bmax[2] + node, z + 1);
            continue;
        }
        if (G == 2 || G == 4) {
            atomicAdd(a.s1[0] + node, (unsigned long long)x);
            atomicAdd(a.s1[1] + node, (unsigned long long)y);
            atomicAdd(a.s1[2] + node, (unsigned long long)z);
        }
        if (G == 4) {
            atomicAdd(a.s2[0] + node, (unsigned long long)x * x);
            atomicAdd(a.s2[1] + node, (unsigned long long)y * y);
            atomicAdd(a.s2[2] + node, (unsigned long long)z * z);
            atomicAdd(a.s2[3] + node, (unsigned long long)x * y);
            atomicAdd(a.s2[4] + node, (unsigned long long)y * z);
            atomicAdd(a.s2[5] + node, (unsigned long long)x * z);
        }
        if (G == 3 || G == 4) {
            const float gv = gval[p];
            if (EXACT) {
                long long gi = (long long)gv;
                atomicAdd((unsigned long long *)a.gw[0] + node, (unsigned long long)gi);
                if (G == 4) atomicAdd((unsigned long long *)a.gw[1] + node, (unsigned long long)(gi * gi));
                atomicAdd((unsigned long long *)a.gw[2] + node, (unsigned long long)(gi * (long long)x));
                atomicAdd((unsigned long long *)a.gw[3] + node, (unsigned long long)(gi * (long long)y));
                atomicAdd((unsigned long long *)a.gw[4] + node, (unsigned long long)(gi * (long long)z));
            } else {
                const double gd = (double)gv;
                atomicAdd((double *)a.gw[0] + node, gd);
                if (G == 4) atomicAdd((double *)a.gw[1] + node, gd * gd);
                atomicAdd((double *)a.gw[2] + node, gd * (double)x);
                atomicAdd((double *)a.gw[3] + node, gd * (double)y);
                atomicAdd((double *)a.gw[4] + node, gd * (double)z);
            }
        }
    }
}

__global__ void k_mark_leaves(long long n, const unsigned char *__restrict__ isroot, int *pending)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x)
        if (isroot[p] && pending[p] == 0) pending[p] = -1;
}

template <int G, bool EXACT>
__device__ __forceinline__ void fold_into(const AttrBufs &a, int u, int q)
{
    atomicAdd(a.area + q, __ldcg(a.area + u));
    if (G == 1) {
        for (int d = 0; d < 3; d++) {
            atomicMin(a.bmin[d] + q, __ldcg(a.bmin[d] + u));
            atomicMax(a.bmax[d] + q, __ldcg(a.bmax[d] + u));
        }
    }
    if (G == 2 || G == 4)
        for (int d = 0; d < 3; d++) atomicAdd(a.s1[d] + q, __ldcg(a.s1[d] + u));
    if (G == 4)
        for (int d = 0; d < 6; d++) atomicAdd(a.s2[d] + q, __ldcg(a.s2[d] + u));
    if (G == 3 || G == 4) {
        for (int d = 0; d < 5; d++) {
            if (G == 3 && d == 1) continue;
            if (EXACT)
                atomicAdd((unsigned long long *)a.gw[d] + q, __ldcg((unsigned long long *)a.gw[d] + u));
            else
                atomicAdd((double *)a.gw[d] + q, __ldcg((double *)a.gw[d] + u));
        }
    }
}

template <int G, bool EXACT>
__global__ void k_attr_up(long long n, const int *__restrict__ parent, AttrBufs a, unsigned *err)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        if (__ldcg(a.pending + p) != -1) continue;
        int u = (int)p;
        long long it = 0;
        for (; it < n; it++) {
            int q = parent[u];
            if (q == NONE) break;
            fold_into<G, EXACT>(a, u, q);
            __threadfence();
            int before = atomicSub(a.pending + q, 1);
            if (before != 1) break;
            __threadfence();
            u = q;
        }
        if (it >= n) raise_error(err, DEVERR_WALK_BOUND);
    }
}

void launch_attributes(const TreeView &t, AttrBufs &a, unsigned *err, int sm, cudaStream_t s)
{
    int nb = grid_for(t.g.N, 256, sm);
#define DCF_PIX(G, E) k_attr_pixels<G, E><<<nb, 256, 0, s>>>(t.gval, t.g, t.parent, t.isroot, a)
    prof_begin(P_ATTR_PIX, s);
    switch (a.group * 2 + (a.exact_g ? 1 : 0)) {
    case 0: case 1: DCF_PIX(0, false); break;
    case 2: case 3: DCF_PIX(1, false); break;
    case 4: case 5: DCF_PIX(2, false); break;
    case 6: DCF_PIX(3, false); break;
    case 7: DCF_PIX(3, true); break;
    case 8: DCF_PIX(4, false); break;
    default: DCF_PIX(4, true); break;
    }
#undef DCF_PIX
    prof_end(P_ATTR_PIX, s);
    prof_begin(P_ATTR_UP, s);
    k_mark_leaves<<<nb, 256, 0, s>>>(t.g.N, t.isroot, a.pending);
#define DCF_UP(G, E) k_attr_up<G, E><<<nb, 256, 0, s>>>(t.g.N, t.parent, a, err)
    switch (a.group * 2 + (a.exact_g ? 1 : 0)) {
    case 0: case 1: DCF_UP(0, false); break;
    case 2: case 3: DCF_UP(1, false); break;
    case 4: case 5: DCF_UP(2, false); break;
    case 6: DCF_UP(3, false); break;
    case 7: DCF_UP(3, true); break;
    case 8: DCF_UP(4, false); break;
    default: DCF_UP(4, true); break;
    }
#undef DCF_UP
    prof_end(P_ATTR_UP, s);
}

__global__ void k_node_attr(Geom g, const unsigned char *__restrict__ isroot, AttrBufs a, int attr, bool area,
                            float pd0, float pd1, float pd2, double *out)
{
    const float pd[3] = {pd0, pd1, pd2};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < g.N;
         p += (long long)gridDim.x * blockDim.x) {
        out[p] = isroot[p] ? (area ? area_value(a, (int)p, pd) : attr_value(a, attr, (int)p, pd))
                           : __longlong_as_double(0x7ff8000000000000LL);
    }
}

void launch_node_attr(const TreeView &t, const AttrBufs &a, int attr, bool area, double *out, int sm,
                      cudaStream_t s)
{
    int nb = grid_for(t.g.N, 256, sm);
    k_node_attr<<<nb, 256, 0, s>>>(t.g, t.isroot, a, attr, area, t.pixdim[0], t.pixdim[1], t.pixdim[2], out);
}

}  // namespace dcf
