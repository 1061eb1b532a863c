// Operations on a built tree (the reference's filtering.c, pattern.c and the
// per-pixel parts of operation.c), re-designed as node-parallel passes:
//
//   k_flag          survive bit of every level root: attribute >= lambda.
//   k_resolve_halving  direct rule (filtering.c:102-154): each node finds its
//                   nearest surviving ancestor-or-self by path halving.
//   k_resolve       max rule (filtering.c:156): nearest kept ancestor-or-self by
//                   walking up; results are written back along the walked path so
//                   later walkers stop early.
//   k_mark_kept     max rule: every survivor marks its ancestors as kept.
//   k_jump_*        pointer jumping over root paths with double buffers: path sums
//                   for the subtractive rule (filtering.c:211-261) and the topmost
//                   removed ancestor for the min rule (filtering.c:55-100).
//   k_filter_out    per pixel: value of its node's resolution, then extract
//                   (gval - out) and min-tree re-inversion (g_max - out),
//                   operation.c:17-28.
//   k_check         per pixel: (float) attribute of its node (filtering.c:47-52).
//   k_spectrum      per level root: dh = gval - gval(parent) in float, bins by
//                   binary search (pattern.c:7-24), dh * area accumulated in a
//                   shared-memory histogram per block, flushed with global atomics.
#include <cstdlib>

#include "dcf_kernels.cuh"
#include "dcf_attr_eval.cuh"

namespace dcf {

constexpr int UNKNOWN = -2;

#define GRID_LOOP(p, n) \
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < (n); p += (long long)gridDim.x * blockDim.x)

// presolve (direct rule): target starts as the forest k_resolve_halving searches, a
// surviving node pointing to itself and any other node to its parent
__global__ void k_flag(Geom g, NodeSet ns, AttrBufs a, int attr, double lambda, float pd0, float pd1, float pd2,
                       const int *__restrict__ parent, unsigned char *flag, int *target, bool presolve)
{
    const float pd[3] = {pd0, pd1, pd2};
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        const bool keep = attr_value(a, attr, (int)p, pd) >= lambda;
        target[p] = !presolve ? UNKNOWN : keep ? p : parent[p];
        flag[p] = keep ? 1 : 0;
    }
}

__global__ void k_mark_kept(Geom g, NodeSet ns, const int *__restrict__ parent,
                            const unsigned char *__restrict__ flag, unsigned *kept, unsigned *err)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        if (!flag[p]) continue;
        int u = (int)p;
        long long it = 0;
        for (; it < g.N && u != NONE; it++) {
            if (atomicExch(kept + u, 1u) == 1u) break;
            u = parent[u];
        }
        if (it >= g.N) raise_error(err, DEVERR_WALK_BOUND);
    }
}

// nearest flagged ancestor-or-self; flag may be a byte array or the kept words
template <typename F>
__global__ void k_resolve(Geom g, NodeSet ns, const int *__restrict__ parent,
                          const F *__restrict__ flag, int *target, unsigned *err)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        if (((volatile int *)target)[p] != UNKNOWN) continue;
        int v = (int)p, res = NONE;
        long long it = 0;
        for (; it < g.N; it++) {
            int t = ((volatile int *)target)[v];
            if (t != UNKNOWN) { res = t; break; }
            if (flag[v]) { res = v; break; }
            int q = parent[v];
            if (q == NONE) { res = NONE; break; }
            v = q;
        }
        if (it >= g.N) raise_error(err, DEVERR_WALK_BOUND);
        for (int w = (int)p; w != v; w = parent[w]) ((volatile int *)target)[w] = res;
        ((volatile int *)target)[v] = res;
    }
}

// Direct rule: nearest surviving ancestor-or-self, by path halving on the forest
// k_flag left in target (survivors point to themselves, other nodes to their
// parent; NONE above an unflagged root).  A walk that ends only after its result is
// known leaves nothing for the nodes it passed, so the nodes of one unflagged chain,
// which sit together in the node list and start together, would each walk the whole
// chain; halving shares every step at once.  Every pointer stays an ancestor at or
// below the nearest survivor, and each node's own thread writes its answer last: a
// halving CAS expects the pointer it read, so a late one cannot replace an answer.
__global__ void k_resolve_halving(Geom g, NodeSet ns, int *target, unsigned *err)
{
    volatile int *tg = target;
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        int v = (int)p, j = tg[v];
        if (j == v) continue;  // survives: its own resolution
        int res = NONE;
        long long it = 0;
        for (; it < g.N; it++) {
            if (j == NONE) break;  // above an unflagged root
            const int jj = tg[j];
            if (jj == j) {  // j survives
                res = j;
                break;
            }
            if (jj == NONE) break;
            atomicCAS(target + v, j, jj);
            v = jj;
            j = tg[v];
            if (j == v) {
                res = v;
                break;
            }
        }
        if (it >= g.N) raise_error(err, DEVERR_WALK_BOUND);
        tg[p] = res;
    }
}

// subtractive: value(u) = sum over the root path of delta(w), delta(w) =
// flag ? gval(w) - gval(parent(w)) : 0, the root's delta being flag ? gval : 0.
__global__ void k_sub_init(Geom g, NodeSet ns, const int *__restrict__ parent,
                           const float *__restrict__ gval, const unsigned char *__restrict__ flag, int *jump,
                           double *acc)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        int q = parent[p];
        jump[p] = q;
        double d = 0.0;
        if (flag[p]) d = q == NONE ? (double)gval[p] : (double)gval[p] - (double)gval[q];
        acc[p] = d;
    }
}

__global__ void k_jump_sum(Geom g, NodeSet ns, const int *__restrict__ jin,
                           const double *__restrict__ ain, int *jout, double *aout)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        int j = jin[p];
        if (j == NONE) {
            jout[p] = NONE;
            aout[p] = ain[p];
        } else {
            jout[p] = jin[j];
            aout[p] = ain[p] + ain[j];
        }
    }
}

// Subtractive rule with the reference's float arithmetic, for images whose levels
// are not small integers: value(u) = (gval(u) + value(w)) - gval(w) for a surviving
// node u under w, value(w) for a removed one, evaluated top-down in float as
// filtering.c:231-243 does.  Each node walks up (at most SUB_STACK steps) to the
// nearest ancestor whose value is known, then evaluates the walked path downward;
// nodes further than that from any known value retry in the next launch.
constexpr int SUB_STACK = 48;

__global__ void k_sub_exact(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent,
                            const float *__restrict__ gval, const unsigned char *__restrict__ flag, float *val,
                            unsigned char *known, unsigned *remaining)
{
    unsigned left = 0;
    GRID_LOOP(p, g.N)
    {
        if (!isroot[p] || ((volatile unsigned char *)known)[p]) continue;
        int stk[SUB_STACK];
        int n = 0, v = (int)p;
        bool have = false, at_root = false;
        while (n < SUB_STACK) {
            if (((volatile unsigned char *)known)[v]) { have = true; break; }
            stk[n++] = v;
            int q = parent[v];
            if (q == NONE) { at_root = true; break; }
            v = q;
        }
        if (!have && !at_root) { left++; continue; }
        __threadfence();  // pairs with the writer's fence between value and flag
        int j = n - 1;
        float above;
        if (at_root) {  // stk[j] is the root
            int r = stk[j];
            above = flag[r] ? gval[r] : 0.0f;
            ((volatile float *)val)[r] = above;
            __threadfence();
            ((volatile unsigned char *)known)[r] = 1;
            j--;
        } else {
            above = ((volatile float *)val)[v];
        }
        for (; j >= 0; j--) {
            int w = stk[j], pw = parent[w];
            float f = flag[w] ? __fsub_rn(__fadd_rn(gval[w], above), gval[pw]) : above;
            ((volatile float *)val)[w] = f;
            __threadfence();
            ((volatile unsigned char *)known)[w] = 1;
            above = f;
        }
    }
    for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
    if ((threadIdx.x & 31) == 0 && left) atomicAdd(remaining, left);
}

// min rule: best(u) = topmost removed node on u's path, root excluded
__global__ void k_min_init(Geom g, NodeSet ns, const int *__restrict__ parent,
                           const unsigned char *__restrict__ flag, int *jump, int *best)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        int q = parent[p];
        jump[p] = q;
        best[p] = (q != NONE && !flag[p]) ? (int)p : NONE;
    }
}

__global__ void k_jump_last(Geom g, NodeSet ns, const int *__restrict__ jin,
                            const int *__restrict__ bin, int *jout, int *bout)
{
    NODE_LOOP(p, ns.nodes, ns.num)
    {
        int j = jin[p];
        if (j == NONE) {
            jout[p] = NONE;
            bout[p] = bin[p];
        } else {
            jout[p] = jin[j];
            int bj = bin[j];
            bout[p] = bj != NONE ? bj : bin[p];
        }
    }
}

// output pixel in the caller's type: float, or (for u8/u16 trees, whose every
// filtered level is an integer in the input's range) the input's own integer type
template <typename O> __device__ __forceinline__ O out_value(float v);
template <> __device__ __forceinline__ float out_value<float>(float v) { return v; }
template <> __device__ __forceinline__ uint16_t out_value<uint16_t>(float v) { return (uint16_t)min(__float2uint_rn(v), 65535u); }
template <> __device__ __forceinline__ uint8_t out_value<uint8_t>(float v) { return (uint8_t)min(__float2uint_rn(v), 255u); }

template <int RULE, typename O>
__global__ void k_filter_out(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent,
                             const float *__restrict__ gval, const unsigned char *__restrict__ flag,
                             const int *__restrict__ target, const double *__restrict__ acc, bool extract,
                             bool tree_min, const unsigned *kmax, O *out)
{
    const float gmax = tree_min ? key_to_level(*kmax) : 0.0f;
    GRID_LOOP(p, g.N)
    {
        const int node = isroot[p] ? (int)p : parent[p];
        float val;
        if (RULE == 0 || RULE == 2) {
            int s = target[node];
            val = s >= 0 ? gval[s] : 0.0f;
        } else if (RULE == 3) {
            val = (float)acc[node];
        } else if (RULE == 4) {
            val = ((const float *)acc)[node];
        } else {  // min
            int r = target[node];
            if (r != NONE) val = gval[parent[r]];
            else if (parent[node] == NONE) val = flag[node] ? gval[node] : 0.0f;
            else val = gval[node];
        }
        if (extract) val = __fsub_rn(gval[p], val);
        if (tree_min) val = __fsub_rn(gmax, val);
        out[p] = out_value<O>(val);
    }
}

static int rounds_for(long long depth_bound)
{
    int r = 0;
    while ((1LL << r) <= depth_bound && r < 40) r++;
    return r;
}

void launch_filter(const TreeView &t, const AttrBufs &a, int attr, int rule, double lambda, bool extract,
                   void *out, const FilterWork &w, long long depth_bound, unsigned *err, int sm, cudaStream_t s,
                   int out_dtype)
{
    const int nb = grid_for(t.g.N, 256, sm);
    prof_begin(P_FLAG, s);
    k_flag<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, a, attr, lambda, t.pixdim[0], t.pixdim[1], t.pixdim[2],
                              t.parent, w.flag, w.target, rule == 0); note_launch();
    prof_end(P_FLAG, s);
    prof_begin(rule == 0 || rule == 2 ? P_RESOLVE : P_JUMP, s);
    const double *accp = nullptr;
    if (rule == 0) {
        k_resolve_halving<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, w.target, err); note_launch();
    } else if (rule == 2) {
        cudaMemsetAsync(w.kept, 0, t.g.N * sizeof(unsigned), s);
        k_mark_kept<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, w.flag, w.kept, err); note_launch();
        k_resolve<unsigned><<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, w.kept, w.target, err); note_launch();
    } else {
        const int R = rounds_for(depth_bound);
        int *j0 = w.jump, *j1 = w.jump2;
        if (rule == 3 && !t.integer_levels) {
            // exact float recurrence, repeated until every node is resolved
            float *val = (float *)w.acc;
            unsigned char *known = (unsigned char *)w.acc2;
            cudaMemsetAsync(known, 0, t.g.N, s);
            for (long long launch = 0; launch <= t.g.N / SUB_STACK + 1; launch++) {
                cudaMemsetAsync(w.remaining, 0, sizeof(unsigned), s);
                k_sub_exact<<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, t.gval, w.flag, val, known, w.remaining); note_launch();
                unsigned left = 0;
                cudaMemcpyAsync(&left, w.remaining, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                if (left == 0) break;
            }
            accp = (const double *)val;
            rule = 4;
        } else if (rule == 3) {
            double *a0 = w.acc, *a1 = w.acc2;
            k_sub_init<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, t.gval, w.flag, j0, a0); note_launch();
            for (int r = 0; r < R; r++) {
                k_jump_sum<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, j0, a0, j1, a1); note_launch();
                int *tj = j0; j0 = j1; j1 = tj;
                double *ta = a0; a0 = a1; a1 = ta;
            }
            accp = a0;
        } else {
            int *b0 = w.target, *b1 = w.best2;
            k_min_init<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, w.flag, j0, b0); note_launch();
            for (int r = 0; r < R; r++) {
                k_jump_last<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, j0, b0, j1, b1); note_launch();
                int *tj = j0; j0 = j1; j1 = tj;
                int *tb = b0; b0 = b1; b1 = tb;
            }
            if (b0 != w.target) cudaMemcpyAsync(w.target, b0, t.g.N * sizeof(int), cudaMemcpyDeviceToDevice, s);
        }
    }
    prof_end(rule == 0 || rule == 2 ? P_RESOLVE : P_JUMP, s);
    prof_begin(P_FILTER_OUT, s);
#define DCF_OUT_T(R, O)                                                                                      \
    {                                                                                                        \
        k_filter_out<R, O><<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, t.gval, w.flag, w.target, accp, extract, \
                                              t.tree_min, t.kmax, (O *)out);                                 \
        note_launch();                                                                                       \
    }
#define DCF_OUT(R)                                            \
    do {                                                      \
        if (out_dtype == U16) DCF_OUT_T(R, uint16_t)          \
        else if (out_dtype == U8) DCF_OUT_T(R, uint8_t)       \
        else DCF_OUT_T(R, float)                              \
    } while (0)
    switch (rule) {
    case 0: DCF_OUT(0); break;
    case 1: DCF_OUT(1); break;
    case 2: DCF_OUT(2); break;
    case 3: DCF_OUT(3); break;
    default: DCF_OUT(4); break;
    }
#undef DCF_OUT
#undef DCF_OUT_T
    prof_end(P_FILTER_OUT, s);
}

__global__ void k_check(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent, AttrBufs a,
                        int attr, float pd0, float pd1, float pd2, float *out)
{
    const float pd[3] = {pd0, pd1, pd2};
    GRID_LOOP(p, g.N)
    {
        const int node = isroot[p] ? (int)p : parent[p];
        out[p] = (float)attr_value(a, attr, node, pd);
    }
}

void launch_check(const TreeView &t, const AttrBufs &a, int attr, float *out, int sm, cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    prof_begin(P_CHECK, s);
    k_check<<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, a, attr, t.pixdim[0], t.pixdim[1], t.pixdim[2], out); note_launch();
    prof_end(P_CHECK, s);
}

// find_scale (pattern.c:7-24): the last bin whose lambda is <= the attribute
__device__ __forceinline__ int find_scale(const float *lv, int n, double v)
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

constexpr int SPEC_SMEM_BINS = 4096;

// ---------------------------------------------------------------------------
// Exact bin search without double arithmetic (GB300 runs FP64 at a small fraction
// of its FP32 rate, and the double readouts and comparisons made the spectrum
// FP64-pipe bound).  With integer levels and unit pixel sizes the binned values
// are exact numbers that can be compared with each float threshold lambda_i
// exactly, so the predicate v >= (double)lambda_i of find_scale -- and therefore
// the bisection's result -- is unchanged:
//   BK_INT    an integer below 2^53 (a group's area readout in groups 1-4, the
//             rectangle area, the x/y/z extents): v >= lambda <=> v >= ceil(lambda);
//   BK_FLOAT  area_attribute with unit pixels is (float) area: compared in float;
//   BK_RATIO  bounding-box elongation hi / max(lo, 1), hi >= lo integers: with
//             lambda = M 2^-S (M its 24-bit mantissa) hi / lo' >= lambda <=>
//             hi 2^S >= M lo' in 64-bit integers.  The double quotient the
//             reference compares falls on the same side of the float threshold:
//             a quotient below lambda is below it by at least 2^-S / lo', more than
//             half an ulp of lambda while lo' <= 2^30 (lo' <= min(W, H) < 2^16 for any
//             image under 2^31 pixels);
//   BK_GENERIC any other attribute: the double readout and comparison.
// ---------------------------------------------------------------------------
enum BinKind : int { BK_GENERIC = 0, BK_INT = 1, BK_FLOAT = 2, BK_RATIO = 3 };
constexpr int SPEC_FAST_MAXBINS = 128;        // thresholds kept in shared memory per vector
constexpr unsigned long long TH_NEVER = ~0ull;

// value kind of binning attribute `attr` (< 0: the group's area readout) of a tree
// of u8/u16 levels with unit pixels
static int bin_kind(int group, int attr)
{
    if (attr < 0) return group == 0 ? BK_FLOAT : BK_INT;
    if (attr == 0) return BK_FLOAT;
    if (group == 1 && (attr == 1 || attr == 3 || attr == 4 || attr == 5)) return BK_INT;
    if (group == 1 && attr == 18) return BK_RATIO;
    return BK_GENERIC;
}

// integer value v >= lambda <=> v >= th (TH_NEVER: never)
__device__ __forceinline__ unsigned long long int_threshold(float lam)
{
    if (lam != lam) return TH_NEVER;
    if (!(lam > 0.0f)) return 0ull;
    const float c = ceilf(lam);
    if (c >= 18446744073709551616.0f) return TH_NEVER;
    return __float2ull_rz(c);
}

// ratio threshold: kind 0 compares hi << s >= m * lo'; 1 always true; 2 never
struct RatioTh {
    unsigned long long m;
    int s;
    int kind;
};
__device__ __forceinline__ RatioTh ratio_threshold(float lam)
{
    RatioTh r{0ull, 0, 2};
    if (lam != lam) return r;                  // NaN: nothing compares >= it
    if (lam <= 1.0f) {                         // every elongation is >= 1
        r.kind = 1;
        return r;
    }
    if (lam >= 2147483648.0f) return r;        // above any hi / lo' (hi < 2^31)
    const unsigned bits = __float_as_uint(lam);
    const int e = (int)((bits >> 23) & 0xFF) - 127;  // lam in [2^e, 2^(e+1)), 0 <= e <= 30
    const unsigned long long mant = (bits & 0x7FFFFFu) | 0x800000u;
    r.kind = 0;
    if (e <= 23) {
        r.m = mant;
        r.s = 23 - e;
    } else {  // lam is the integer mant * 2^(e-23)
        r.m = mant << (e - 23);
        r.s = 0;
    }
    return r;
}

__device__ __forceinline__ bool ratio_ge(unsigned hi, unsigned lo1, const RatioTh &t)
{
    if (t.kind != 0) return t.kind == 1;
    return ((unsigned long long)hi << t.s) >= t.m * (unsigned long long)lo1;
}

// the bisection of find_scale (pattern.c:7-24) over a predicate ge(i) = "value >= lambda_i"
template <class GE>
__device__ __forceinline__ int find_scale_pred(int n, GE ge)
{
    int upper = n - 1, lower = 0;
    if (ge(upper)) return upper;
    int mid = (upper + lower) / 2;
    while (mid != lower) {
        if (ge(mid)) lower = mid;
        else upper = mid;
        mid = (upper + lower) / 2;
    }
    return lower;
}

struct BinTh {
    unsigned long long it[SPEC_FAST_MAXBINS];
    RatioTh rt[SPEC_FAST_MAXBINS];
};

// bin of node u on lambda vector lv (n values) for a value of kind `kind` != BK_GENERIC
__device__ __forceinline__ int fast_bin(const AttrBufs &a, int attr, int kind, int u, const float *lv, int n,
                                        const BinTh &th)
{
    if (kind == BK_INT) {
        unsigned long long v;
        if (attr < 0) v = a.area[u];
        else if (attr == 1)
            v = (unsigned long long)(a.bmax[0][u] - a.bmin[0][u]) * (a.bmax[1][u] - a.bmin[1][u]) *
                (a.bmax[2][u] - a.bmin[2][u]);
        else v = a.bmax[attr - 3][u] - a.bmin[attr - 3][u];
        return find_scale_pred(n, [&](int i) { return th.it[i] != TH_NEVER && v >= th.it[i]; });
    }
    if (kind == BK_FLOAT) {
        const float f = __uint2float_rn(a.area[u]);
        return find_scale_pred(n, [&](int i) { return f >= lv[i]; });
    }
    const unsigned xe = a.bmax[0][u] - a.bmin[0][u], ye = a.bmax[1][u] - a.bmin[1][u];
    const unsigned hi = xe > ye ? xe : ye, lo = xe < ye ? xe : ye, lo1 = lo > 1u ? lo : 1u;
    return find_scale_pred(n, [&](int i) { return ratio_ge(hi, lo1, th.rt[i]); });
}

// EXACT: u8/u16 levels and unit pixel sizes, so every dh * area is an integer below
// 2^48 and every bin's sum is below 2^53 (the sum of all bins is the image's grey
// sum): any summation order gives the reference's double sums bit for bit.  The
// lanes of a warp that hit one bin then add their terms first (three 22-bit limbs,
// one __reduce_add_sync each) and their leader issues one shared-memory 64-bit
// integer atomic; otherwise every node adds its double term on its own.
template <bool EXACT>
__global__ void __launch_bounds__(256, 3) k_spectrum(Geom g, NodeSet ns, const int *__restrict__ parent,
                           const float *__restrict__ gval, AttrBufs a, int a1, const float *__restrict__ l1, int n1,
                           int a2, const float *__restrict__ l2, int n2, float pd0, float pd1, float pd2,
                           double *spec, int k1, int k2)
{
    __shared__ double hist[SPEC_SMEM_BINS];
    unsigned long long *ihist = (unsigned long long *)hist;
    const int nbins = n1 * n2;
    const bool priv = nbins <= SPEC_SMEM_BINS;
    if (priv)
        for (int i = threadIdx.x; i < nbins; i += blockDim.x) hist[i] = 0.0;
    __syncthreads();
    const float pd[3] = {pd0, pd1, pd2};
    if (EXACT) {
        // thresholds of both lambda vectors for the exact-arithmetic bin search (BinKind)
        __shared__ BinTh th[2];
        for (int i = threadIdx.x; i < SPEC_FAST_MAXBINS; i += blockDim.x) {
            if (k1 != BK_GENERIC && i < n1) {
                th[0].it[i] = int_threshold(l1[i]);
                th[0].rt[i] = ratio_threshold(l1[i]);
            }
            if (k2 != BK_GENERIC && i < n2) {
                th[1].it[i] = int_threshold(l2[i]);
                th[1].rt[i] = ratio_threshold(l2[i]);
            }
        }
        __syncthreads();
        const int lane = threadIdx.x & 31;
        const long long wstride = (long long)gridDim.x * blockDim.x;
        const long long m = (long long)*ns.num;
        // whole warps iterate together so the match below sees the full warp
        for (long long base = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane; base < m;
             base += wstride) {
            const int p = base + lane < m ? ns.nodes[base + lane] : NONE;
            int bin = -1;
            unsigned long long v = 0;
            if (p != NONE) {
                const int q = parent[p];
                const float dh = q != NONE ? __fsub_rn(gval[p], gval[q]) : gval[p];
                if (dh != 0.0f) {
                    const int s1 = k1 != BK_GENERIC ? fast_bin(a, a1, k1, p, l1, n1, th[0])
                                                    : find_scale(l1, n1, a1 < 0 ? area_value(a, p, pd)
                                                                                : attr_value(a, a1, p, pd));
                    const int s2 = n2 <= 1             ? 0
                                   : k2 != BK_GENERIC ? fast_bin(a, a2, k2, p, l2, n2, th[1])
                                                      : find_scale(l2, n2, a2 < 0 ? area_value(a, p, pd)
                                                                                  : attr_value(a, a2, p, pd));
                    bin = s1 + s2 * n1;
                    // dh times the group's area readout, both integers (group 0 reads
                    // the area through float, an integer too)
                    const unsigned ar = a.group == 0 ? __float2uint_rn(__uint2float_rn(a.area[p])) : a.area[p];
                    v = (unsigned long long)__float2uint_rn(dh) * ar;
                }
            }
            const unsigned grp = __match_any_sync(0xffffffffu, bin);
            if (bin < 0) continue;
            const unsigned long long lo = __reduce_add_sync(grp, (unsigned)(v & 0x3FFFFFu));
            const unsigned long long mid = __reduce_add_sync(grp, (unsigned)((v >> 22) & 0x3FFFFFu));
            const unsigned long long hi = __reduce_add_sync(grp, (unsigned)(v >> 44));
            if (lane != __ffs(grp) - 1) continue;
            const unsigned long long sum = lo + (mid << 22) + (hi << 44);
            if (priv) atomicAdd(ihist + bin, sum);
            else atomicAdd(spec + bin, (double)sum);
        }
    } else {
        NODE_LOOP(p, ns.nodes, ns.num)
        {
            const int q = parent[p];
            const float dh = q != NONE ? __fsub_rn(gval[p], gval[q]) : gval[p];
            if (dh == 0.0f) continue;
            const double ar = area_value(a, (int)p, pd);
            const int s1 = find_scale(l1, n1, a1 < 0 ? ar : attr_value(a, a1, (int)p, pd));
            const int s2 = n2 <= 1 ? 0 : find_scale(l2, n2, a2 < 0 ? ar : attr_value(a, a2, (int)p, pd));
            const double v = (double)dh * ar;
            if (priv) atomicAdd(hist + s1 + s2 * n1, v);
            else atomicAdd(spec + s1 + s2 * n1, v);
        }
    }
    if (!priv) return;
    __syncthreads();
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) {
        if (EXACT) {
            if (ihist[i] != 0) atomicAdd(spec + i, (double)ihist[i]);
        } else if (hist[i] != 0.0) {
            atomicAdd(spec + i, hist[i]);
        }
    }
}

void launch_spectrum(const TreeView &t, const AttrBufs &a, int a1, const float *l1, int n1, int a2, const float *l2,
                     int n2, double *spec, int sm, cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    const bool exact = t.integer_levels && t.pixdim[0] == 1.0f && t.pixdim[1] == 1.0f && t.pixdim[2] == 1.0f;
    // the exact-arithmetic bin search, per lambda vector (BinKind); DCF_SPEC_FP64=1 in
    // the environment keeps the double search (for timing comparisons)
    static const bool fp64 = [] {
        const char *e = getenv("DCF_SPEC_FP64");
        return e && atoi(e) != 0;
    }();
    const int k1 = exact && !fp64 && n1 <= SPEC_FAST_MAXBINS ? bin_kind(a.group, a1) : BK_GENERIC;
    const int k2 = exact && !fp64 && n2 <= SPEC_FAST_MAXBINS ? bin_kind(a.group, a2) : BK_GENERIC;
    prof_begin(P_SPECTRUM, s);
    if (exact)
        k_spectrum<true><<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, t.gval, a, a1, l1, n1, a2,
                                            l2, n2, t.pixdim[0], t.pixdim[1], t.pixdim[2], spec, k1, k2);
    else
        k_spectrum<false><<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, t.parent, t.gval, a, a1, l1, n1, a2,
                                             l2, n2, t.pixdim[0], t.pixdim[1], t.pixdim[2], spec, k1, k2);
    note_launch();
    prof_end(P_SPECTRUM, s);
}

// ---------------------------------------------------------------------------
// CSL segmentation (node_differential_seg, csl.c:27-124): for every node, along its
// root path, the largest run of contrast (summed dh) within one scale class, the
// scale class it was found in and the grey level where it peaked.  State of a
// level root u: maxScale, maxDH, maxOrig, curScale, curDH.  A node whose scale is
// past the last lambda, or the root, restarts the state; any other node extends its
// parent's state with dh(u).  Evaluated like the exact subtractive rule: each node
// walks up (at most CSL_STACK steps) to a node whose state is known or that
// restarts, then evaluates the walked path downward; the rest retry next launch.
// ---------------------------------------------------------------------------
constexpr int CSL_STACK = 48;

// find_scale_csl (csl.c:9-25): past the last lambda -> n (one beyond the bins)
__device__ __forceinline__ int find_scale_csl(const float *lv, int n, double v)
{
    int upper = n - 1, lower = 0;
    if (v >= (double)lv[upper]) return upper + 1;
    int mid = (upper + lower) / 2;
    while (mid != lower) {
        if (v >= (double)lv[mid]) lower = mid;
        else upper = mid;
        mid = (upper + lower) / 2;
    }
    return lower;
}

struct CslState {
    int *max_scale, *cur_scale, *my_scale;
    float *max_dh, *max_orig, *cur_dh;
    unsigned char *known;
};

__global__ void k_csl_init(Geom g, const unsigned char *__restrict__ isroot, AttrBufs a, int attr,
                           const float *__restrict__ lv, int n, float pd0, float pd1, float pd2, CslState c)
{
    const float pd[3] = {pd0, pd1, pd2};
    GRID_LOOP(p, g.N)
    {
        c.known[p] = 0;
        if (isroot[p]) c.my_scale[p] = find_scale_csl(lv, n, attr_value(a, attr, (int)p, pd));
    }
}

__global__ void k_csl(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent,
                      const float *__restrict__ gval, int n, CslState c, unsigned *remaining)
{
    unsigned left = 0;
    GRID_LOOP(p, g.N)
    {
        if (!isroot[p] || ((volatile unsigned char *)c.known)[p]) continue;
        int stk[CSL_STACK];
        int depth = 0, v = (int)p;
        bool have = false, restart = false;
        while (depth < CSL_STACK) {
            if (((volatile unsigned char *)c.known)[v]) { have = true; break; }
            stk[depth++] = v;
            if (parent[v] == NONE || c.my_scale[v] == n) { restart = true; break; }
            v = parent[v];
        }
        if (!have && !restart) { left++; continue; }
        __threadfence();  // pairs with the writer's fence between state and flag
        int ms, cs;
        float mdh, mo, cdh;
        int j = depth - 1;
        if (restart) {  // stk[j] starts a state of its own
            const int r = stk[j];
            const bool root = parent[r] == NONE;
            ms = root ? c.my_scale[r] : n;
            mo = root ? gval[r] : 0.0f;
            mdh = 0.0f;
            cdh = 0.0f;
            cs = ms;
        } else {
            ms = ((volatile int *)c.max_scale)[v];
            cs = ((volatile int *)c.cur_scale)[v];
            mdh = ((volatile float *)c.max_dh)[v];
            mo = ((volatile float *)c.max_orig)[v];
            cdh = ((volatile float *)c.cur_dh)[v];
            j = depth;  // every stacked node extends a known state
        }
        for (int k = restart ? j : j - 1; k >= 0; k--) {
            const int w = stk[k];
            if (!(restart && k == j)) {
                const int sw = c.my_scale[w];
                const float dh = __fsub_rn(gval[w], gval[parent[w]]);
                if (sw == cs) cdh = __fadd_rn(cdh, dh);
                else {
                    cdh = dh;
                    cs = sw;
                }
                if (cdh >= mdh) {
                    mdh = cdh;
                    ms = cs;
                    mo = gval[w];
                }
            }
            ((volatile int *)c.max_scale)[w] = ms;
            ((volatile int *)c.cur_scale)[w] = cs;
            ((volatile float *)c.max_dh)[w] = mdh;
            ((volatile float *)c.max_orig)[w] = mo;
            ((volatile float *)c.cur_dh)[w] = cdh;
            __threadfence();
            ((volatile unsigned char *)c.known)[w] = 1;
        }
    }
    for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(0xffffffffu, left, o);
    if ((threadIdx.x & 31) == 0 && left) atomicAdd(remaining, left);
}

__global__ void k_csl_out(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent, CslState c,
                          float *contrast, float *scale, float *luminance)
{
    GRID_LOOP(p, g.N)
    {
        const int u = isroot[p] ? (int)p : parent[p];
        contrast[p] = c.max_dh[u];
        scale[p] = (float)c.max_scale[u];
        luminance[p] = c.max_orig[u];
    }
}

// the seven arrays launch_csl carves, each rounded up to 256 bytes (so that what a
// caller places after them stays 256-byte aligned)
size_t csl_work_bytes(long long n)
{
    const size_t a4 = ((size_t)n * 4 + 255) / 256 * 256, a1 = ((size_t)n + 255) / 256 * 256;
    return 6 * a4 + a1;
}

void launch_csl(const TreeView &t, const AttrBufs &a, int attr, const float *lv, int n, float *contrast, float *scale,
                float *luminance, void *work, unsigned *remaining, int sm, cudaStream_t s)
{
    const long long N = t.g.N;
    char *m = (char *)work;
    auto take = [&](size_t b) { void *p = m; m += (b + 255) / 256 * 256; return p; };
    CslState c;
    c.max_scale = (int *)take(4 * N);
    c.cur_scale = (int *)take(4 * N);
    c.my_scale = (int *)take(4 * N);
    c.max_dh = (float *)take(4 * N);
    c.max_orig = (float *)take(4 * N);
    c.cur_dh = (float *)take(4 * N);
    c.known = (unsigned char *)take(N);
    const int nb = grid_for(N, 256, sm);
    k_csl_init<<<nb, 256, 0, s>>>(t.g, t.isroot, a, attr, lv, n, t.pixdim[0], t.pixdim[1], t.pixdim[2], c);
    note_launch();
    for (long long launch = 0; launch <= N / CSL_STACK + 1; launch++) {
        cudaMemsetAsync(remaining, 0, sizeof(unsigned), s);
        k_csl<<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, t.gval, n, c, remaining);
        note_launch();
        unsigned left = 0;
        cudaMemcpyAsync(&left, remaining, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        if (left == 0) break;
    }
    k_csl_out<<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, c, contrast, scale, luminance);
    note_launch();
}

// ---------------------------------------------------------------------------
// adjoint (no reference counterpart)
// ---------------------------------------------------------------------------
// With the tree fixed, the direct-rule output out(p) = level(target(node(p))) and
// the spectrum term dh(u) * area(u), dh(u) = level(u) - level(parent(u)), are
// linear in the levels; a node's level is the value of its level root pixel.  So
//   d loss / d level(s) += v(p)                       for target(node(p)) = s,
//   d loss / d level(u) += w(bin(u)) * area(u),  d loss / d level(parent(u)) -= same.
__device__ __forceinline__ int cutout_of(const long long *offs, int count, long long p)
{
    int lo = 0, hi = count - 1;  // last cutout whose first pixel is <= p
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (offs[mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_adjoint(Geom g, const unsigned char *__restrict__ isroot, const int *__restrict__ parent,
                          AttrBufs a, AdjointArgs j, float pd0, float pd1, float pd2)
{
    const float pd[3] = {pd0, pd1, pd2};
    GRID_LOOP(p, g.N)
    {
        const bool root = isroot[p];
        if (j.target) {
            const int s = j.target[root ? (int)p : parent[p]];
            if (s >= 0) atomicAdd(j.acc + s, (double)j.v[p]);
        }
        if (!j.w || !root) continue;
        const double ar = area_value(a, (int)p, pd);
        const int s1 = find_scale(j.l1, j.n1, j.a1 < 0 ? ar : attr_value(a, j.a1, (int)p, pd));
        const int s2 = j.n2 <= 1 ? 0 : find_scale(j.l2, j.n2, j.a2 < 0 ? ar : attr_value(a, j.a2, (int)p, pd));
        const int img = j.count > 1 ? cutout_of(j.offs, j.count, p) : 0;
        const double c = j.w[(long long)img * j.n1 * j.n2 + s1 + s2 * j.n1] * ar;
        if (c == 0.0) continue;
        atomicAdd(j.acc + p, c);
        const int q = parent[p];
        if (q != NONE) atomicAdd(j.acc + q, -c);
    }
}

__global__ void k_adjoint_out(long long n, const double *__restrict__ acc, float *grad)
{
    GRID_LOOP(p, n) grad[p] = (float)acc[p];
}

void launch_adjoint(const TreeView &t, const AttrBufs &a, const AdjointArgs &j, int sm, cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    prof_begin(P_ADJOINT, s);
    k_adjoint<<<nb, 256, 0, s>>>(t.g, t.isroot, t.parent, a, j, t.pixdim[0], t.pixdim[1], t.pixdim[2]); note_launch();
    k_adjoint_out<<<nb, 256, 0, s>>>(t.g.N, j.acc, j.grad); note_launch();
    prof_end(P_ADJOINT, s);
}

// direct rule without the output pass: survive flags and resolved targets
void launch_direct_targets(const TreeView &t, const AttrBufs &a, int attr, double lambda, const FilterWork &w,
                           unsigned *err, int sm, cudaStream_t s)
{
    const int nb = grid_for(t.g.N, 256, sm);
    prof_begin(P_FLAG, s);
    k_flag<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, a, attr, lambda, t.pixdim[0], t.pixdim[1], t.pixdim[2],
                              t.parent, w.flag, w.target, true); note_launch();
    prof_end(P_FLAG, s);
    prof_begin(P_RESOLVE, s);
    k_resolve_halving<<<nb, 256, 0, s>>>(t.g, NodeSet{t.nodes, t.num_nodes}, w.target, err); note_launch();
    prof_end(P_RESOLVE, s);
}

}  // namespace dcf
