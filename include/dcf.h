/*
 * dcf.h -- C ABI of the GB300 component-forest library (libdcf_gb300.so).
 *
 * Drop-in for the hot path of disccofan: max/min-tree construction, attribute
 * accumulation, attribute filtering and pattern spectra.  Plain C types only; every
 * call returns a dcf_status.  Pixels are in x-fastest order (index = x + y*W +
 * z*W*H), the same order the reference's Node.gval uses.  A pointer argument is a
 * HOST pointer unless the call's on_device flag says it is a device pointer.
 *
 * Reference interfaces each call replaces (paths relative to the reference repo):
 *   dcf_tree_build            build_tree_with_attributes      src/sources/flood.c:175
 *                             (with preprocessing's min-tree inversion,
 *                              src/sources/preprocessing.c:77-91, and io.c:64-79's
 *                              connectivity fix-ups)
 *   dcf_tree_set_attribute    flood_attributes                src/sources/flood.c:184
 *   dcf_tree_parent           Node.parent after the build (types.h:147-159) /
 *                             get_levelroot                   src/sources/flood.c:693
 *   dcf_node_attribute        AttribsArray[i].attribute/.area src/sources/attributes.c:1224
 *   dcf_filter                tree_filtering + perform_filter_or_extract
 *                                                             src/sources/filtering.c:18,
 *                                                             src/sources/operation.c:10
 *   dcf_attribute_check       tree_attribute_check            src/sources/filtering.c:47
 *   dcf_pattern_spectrum      tree_pattern_spectrum           src/sources/pattern.c:27
 *   dcf_pattern_spectrum2d    tree_pattern_spectrum2d (+ the attribute-order rule of
 *                             perform_pattern_spectrum)       src/sources/pattern.c:110,
 *                                                             src/sources/operation.c:88-100
 *   dcf_dmp                   perform_dmp_operation           src/sources/operation.c:63
 *   dcf_csl                   perform_csl / tree_differential src/sources/operation.c:31,
 *                                                             src/sources/csl.c:27-146
 *   dcf_lvec_read             lambda_vector_read              src/sources/lambdavec.c:35
 *   dcf_tree_export           write_tree                      src/sources/io.c:1431
 *   dcf_fits_read             the FITS branch of the tile reader src/sources/io.c:624-706
 *   dcf_fits_read_raw         (same, in the file's own pixel type)
 *   dcf_batch_*               (no reference counterpart: many cutouts per launch)
 *   dcf_adjoint_*             (no reference counterpart: gradients for float images)
 */
#ifndef DCF_H
#define DCF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DCF_OK = 0,
    DCF_ERR_INVALID = 1,     /* bad argument (dims, connectivity, attribute, rule, sizes) */
    DCF_ERR_NOMEM = 2,       /* device or host allocation failed */
    DCF_ERR_CUDA = 3,        /* a CUDA call failed; dcf_ctx_last_error has the text */
    DCF_ERR_TIMEOUT = 4,     /* a bounded device loop gave up (merge/walk/wait bound) */
    DCF_ERR_NAN = 5,         /* the image holds NaN: its grey levels are unordered */
    DCF_ERR_STATE = 6,       /* call not valid in the object's current state */
    DCF_ERR_IO = 7,          /* file could not be read or parsed */
    DCF_ERR_UNSUPPORTED = 8  /* valid request this build does not implement */
} dcf_status;

typedef enum { DCF_U8 = 0, DCF_U16 = 1, DCF_U32 = 2, DCF_F32 = 3 } dcf_dtype;
typedef enum { DCF_MAX_TREE = 0, DCF_MIN_TREE = 1 } dcf_tree_type;
/* filter rules, in the reference's Decisions[] order (filtering.c:271-277) */
typedef enum { DCF_RULE_DIRECT = 0, DCF_RULE_MIN = 1, DCF_RULE_MAX = 2, DCF_RULE_SUBTRACTIVE = 3 } dcf_rule;

/* Attribute indices 0..17 are the reference's AttribsArray (attributes.c:1224-1248):
 * 0 area | 1 rectarea 2 rectdiag 3 xext 4 yext 5 zext | 6 xmean 7 ymean 8 zmean |
 * 9 xwmean 10 ywmean 11 zwmean 12 flux | 13 inertia trace 14 elongation 15 flatness
 * 16 sparseness 17 non-compactness.  18 = bounding-box elongation
 * max(xext,yext)/max(min(xext,yext),1) on the extent group (not in the reference). */
#define DCF_NUM_ATTRIBUTES 19

typedef struct dcf_ctx dcf_ctx;
typedef struct dcf_tree dcf_tree;

typedef struct {
    const void *data;        /* pixels, x fastest */
    int dtype;               /* dcf_dtype */
    int on_device;           /* 1: data is a device pointer on the context's device */
    uint64_t dims[3];        /* width, height, depth (depth = 1 for 2-D) */
    int connectivity;        /* 4 or 8 (2-D), 6 or 26 (3-D); fixed up like io.c:64-79 */
    int tree_type;           /* dcf_tree_type */
    float pixdim[3];         /* physical pixel size (config pixel_dim); 1,1,1 usual */
} dcf_image;

/* ---- context: one device, one stream, a reusable device workspace ---- */
dcf_status dcf_ctx_create(int device, void *cuda_stream, dcf_ctx **out);
dcf_status dcf_ctx_destroy(dcf_ctx *ctx);
dcf_status dcf_ctx_synchronize(dcf_ctx *ctx);
const char *dcf_ctx_last_error(const dcf_ctx *ctx);
const char *dcf_status_string(dcf_status s);
/* number of device kernel launches issued through this context so far */
uint64_t dcf_ctx_launch_count(const dcf_ctx *ctx);
/* The cudaStream_t every call of this context is ordered on (the one given to
 * dcf_ctx_create, else one the context created, non-blocking).  Device buffers a
 * call reads must be ready on it, and device outputs are complete only in its
 * order: a caller producing or consuming them on another stream orders the two
 * (an event, or cudaStreamWaitEvent). */
void *dcf_ctx_stream(const dcf_ctx *ctx);

/* Per-kernel timing with CUDA events on the context's stream (0 = off).  Turning
 * it on or off resets the totals; dcf_ctx_profile returns the summed device time
 * and launch-group count of kernel `id` (0 <= id < dcf_profile_num_kernels()). */
dcf_status dcf_ctx_set_profiling(dcf_ctx *ctx, int enable);
dcf_status dcf_ctx_profile(dcf_ctx *ctx, int id, double *total_ms, uint64_t *launches);
int dcf_profile_num_kernels(void);
const char *dcf_profile_kernel_name(int id);

/* ---- tree ---- */
/* Build the max-tree (min-tree: of the inverted image) with the attribute group
 * of attr_idx.  The image is copied to the device when on_device == 0. */
dcf_status dcf_tree_build(dcf_ctx *ctx, const dcf_image *img, int attr_idx, dcf_tree **out);
/* Copy a host image to the context's device staging buffer once, for several
 * builds from the same pixels (the max- and the min-tree of one image): *out is
 * *in with data pointing at the staged copy and on_device = 1.  The copy is
 * ordered on the context's stream; the staged image stays valid until the next
 * dcf_image_stage on this context or its destruction.  An image already on the
 * device is returned unchanged.  (No reference counterpart: the reference reads
 * its input once into Node.gval.) */
dcf_status dcf_image_stage(dcf_ctx *ctx, const dcf_image *in, dcf_image *out);
/* Accumulate the attribute group of attr_idx on the existing tree (no rebuild). */
dcf_status dcf_tree_set_attribute(dcf_ctx *ctx, dcf_tree *tree, int attr_idx);
dcf_status dcf_tree_destroy(dcf_tree *tree);
dcf_status dcf_tree_info(const dcf_tree *tree, uint64_t *num_pixels, uint64_t *num_nodes, int *connectivity,
                         float *max_gval);
/* Canonical parent array: a pixel that is not a level root -> its node's level
 * root (the lowest index of the node's flat zone); a level root -> its parent
 * node's level root; the root -> -1.  Bit-identical to the reference's
 * sequential Node.parent after build_tree_with_attributes. */
dcf_status dcf_tree_parent(dcf_ctx *ctx, dcf_tree *tree, int64_t *parent, int on_device);
/* Grey levels the tree was built on (float; inverted for a min-tree). */
dcf_status dcf_tree_gval(dcf_ctx *ctx, dcf_tree *tree, float *gval, int on_device);
/* Attribute (area=0) or group area readout (area=1) of every level root; NaN at
 * other pixels.  attr_idx must belong to the tree's current attribute group. */
dcf_status dcf_node_attribute(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, int area, double *out, int on_device);

/* ---- operations ---- */
/* tree_filtering with rule, then extract (gval - out) when extract != 0, then the
 * min-tree re-inversion g_max - out.  out: width*height*depth floats. */
dcf_status dcf_filter(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, int rule, double lambda, int extract,
                      float *out, int on_device);
/* dcf_filter with the output in out_dtype: DCF_F32, or, for a tree of a DCF_U8 /
 * DCF_U16 image, that same type -- every filtered value of such an image is an
 * integer of its range, and the reference writes 8/16-bit outputs in the input's
 * depth (write_basic, io.c:1802-1841) -- which halves or quarters the bytes read
 * back.  Other types: DCF_ERR_INVALID. */
dcf_status dcf_filter_as(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, int rule, double lambda, int extract,
                         int out_dtype, void *out, int on_device);
/* out[p] = (float) attribute of p's node. */
dcf_status dcf_attribute_check(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, float *out, int on_device);
/* Differential morphological profile: for each lvec[i+1], i < num_lambdas-1,
 * out[i*N + p] = gval - filter(lvec[i+1]). */
dcf_status dcf_dmp(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, int rule, const float *lvec, int num_lambdas,
                   float *out, int on_device);
/* 1-D pattern spectrum; lvec holds num_lambdas bins INCLUDING the leading 0 (the
 * output of dcf_lvec_read).  spectrum[num_lambdas] is ACCUMULATED (+=), as the
 * reference accumulates into a caller-zeroed array (pattern.c:98-105). */
dcf_status dcf_pattern_spectrum(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, const float *lvec, int num_lambdas,
                                double *spectrum, int on_device);
/* 2-D pattern spectrum, spectrum[s1 + s2*n1] accumulated.  As in the reference,
 * attr1 must be the higher index unless attr2 is 0, and attr2 == 0 bins by the
 * first attribute group's area. */
dcf_status dcf_pattern_spectrum2d(dcf_ctx *ctx, dcf_tree *tree, int attr1, const float *lvec1, int n1, int attr2,
                                  const float *lvec2, int n2, double *spectrum, int on_device);

/* Direct-rule filter (dcf_filter with rule DCF_RULE_DIRECT) that allocates
 * nothing.  No counterpart in the reference: it exists for callers that cannot
 * allocate device memory while filtering -- a host framework whose caching
 * allocator already holds the device's free memory, or a real-time loop that must
 * not wait on or fail in an allocation.  Its per-pixel scratch is a fixed 40 MiB
 * device array inside the library (held by every GPU that loads it until exit), so
 * the tree may have at most 8,388,608 pixels (DCF_ERR_INVALID beyond that).
 * out_device must be device memory, and the tree must be on the context's device.
 * The first call on a device looks up the array's device address (then cached
 * for the life of the process: a caller that resets the device must not call it
 * again); make that first call before any stream capture.  All
 * calls share the one array: calls that overlap on the GPU (other streams or
 * contexts) race and must not be issued concurrently. */
dcf_status dcf_filter_direct_noalloc(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, double lambda, int extract,
                                     float *out_device);

/* ---- batches of 2-D cutouts, and the adjoint (no reference counterparts) ---- */
typedef struct dcf_batch dcf_batch;

/* Operations of a batch run (and of dcf_tree_adjoint).  filter_attr >= 0: the
 * direct-rule filter (keep nodes whose attribute >= lambda; max-tree, no
 * extract).  spec_attr1 >= 0: a 2-D pattern spectrum per cutout with the
 * argument rules of dcf_pattern_spectrum2d (spec_attr2 = 0 bins by area; n2 = 1
 * with lvec2 = {0} gives a 1-D spectrum).  lvec1/lvec2 are host arrays that
 * include the leading 0.  use_graph = 1: the device work of a run is recorded as
 * one CUDA graph (on the second run; the first learns a buffer capacity) and
 * replayed while the pointers and operations stay the same. */
typedef struct {
    int filter_attr;
    double lambda;
    int spec_attr1;
    const float *lvec1;
    int n1;
    int spec_attr2;
    const float *lvec2;
    int n2;
    int use_graph;
} dcf_op_set;

/* A batch of `count` 2-D cutouts of one dtype, widths[i] x heights[i] pixels,
 * built as max-trees with connectivity 4 or 8 and the attribute group of
 * attr_idx.  Pixels are concatenated: cutout i starts at element sum_{j<i}
 * widths[j]*heights[j] (x fastest inside a cutout); at most 2^31-1 in total.
 * Every device buffer is allocated here (or on the first run needing it).
 * Destroy batches before their context. */
dcf_status dcf_batch_create(dcf_ctx *ctx, int count, const uint32_t *widths, const uint32_t *heights, int dtype,
                            int connectivity, int attr_idx, const float *pixdim, dcf_batch **out);
dcf_status dcf_batch_destroy(dcf_batch *batch);
/* schedule[6] = tile width, tile height, CTAs per SM, tiles per queue grab, seam
 * buckets, bottom-up steps; graph_kernels = kernel nodes of the last graph launched */
dcf_status dcf_batch_info(const dcf_batch *batch, uint64_t *total_pixels, uint64_t *num_nodes, int *schedule,
                          uint64_t *graph_kernels);
/* Persistent tile-build schedule (ctas_per_sm <= 0: as many as fit). */
dcf_status dcf_batch_set_schedule(dcf_ctx *ctx, dcf_batch *batch, int tile_w, int tile_h, int ctas_per_sm, int chunk);
/* Tree-merge parameters: seam_buckets = number of ascending-level ranges the seam
 * edges are merged in (0 = all at once; at most 256); up_steps = bottom-up fold
 * steps per walker before the remaining nodes are finished by pointer jumping. */
dcf_status dcf_batch_set_merge(dcf_ctx *ctx, dcf_batch *batch, int seam_buckets, int up_steps);
/* Time, on these pixels, the build over tile shapes, then CTAs per SM and queue
 * chunk for the best shape, then seam buckets, then build + attributes over
 * bottom-up steps; keep the fastest of each.  Leaves no valid trees. */
dcf_status dcf_batch_autotune(dcf_ctx *ctx, dcf_batch *batch, const void *pixels, int on_device, int repeats,
                              double *best_ms);
/* Build every cutout's tree and attributes, then the requested operations:
 * filtered (N floats, may be NULL) and spectra (count * n1 * n2 doubles,
 * spectra[i*n1*n2 + s1 + s2*n1], OVERWRITTEN; may be NULL).  With
 * outputs_on_device = 0 both are host arrays. */
dcf_status dcf_batch_run(dcf_ctx *ctx, dcf_batch *batch, const void *pixels, int pixels_on_device,
                         const dcf_op_set *ops, float *filtered, double *spectra, int outputs_on_device);
/* Canonical parents of the last run, as indices inside each cutout (-1: root). */
dcf_status dcf_batch_parent(dcf_ctx *ctx, dcf_batch *batch, int64_t *parent, int on_device);
/* Attribute of every level root of the last run (NaN elsewhere). */
dcf_status dcf_batch_node_attribute(dcf_ctx *ctx, dcf_batch *batch, int attr_idx, double *out, int on_device);
/* Adjoint of the last run's operations with its trees held fixed (float32
 * pixels): grad_pixels = d loss / d pixels for loss = sum(grad_filtered *
 * filtered) + sum(grad_spectra * spectra).  Either cotangent may be NULL.  A
 * node's level is its level root's pixel value, so each node's terms land on
 * that pixel. */
dcf_status dcf_batch_adjoint(dcf_ctx *ctx, dcf_batch *batch, const float *grad_filtered, const double *grad_spectra,
                             float *grad_pixels, int on_device);
/* The same adjoint for one tree (a float32 max-tree) and the operations in ops. */
dcf_status dcf_tree_adjoint(dcf_ctx *ctx, dcf_tree *tree, const dcf_op_set *ops, const float *grad_filtered,
                            const double *grad_spectrum, float *grad_pixels, int on_device);

/* CSL segmentation (perform_csl operation.c:31, node_differential_seg
 * csl.c:27-124; the reference implements only this first part): per pixel, along
 * its node's root path, the largest contrast (dh summed within one scale class of
 * attr_idx on the lambda bins lvec, num_lambdas values with the leading 0), the
 * scale class it was found in and the grey level where it peaked.  Three
 * width*height*depth float images. */
dcf_status dcf_csl(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, const float *lvec, int num_lambdas, float *contrast,
                   float *scale, float *luminance, int on_device);

/* ---- files ---- */
/* Write the tree in the reference's tree-file format (write_tree, io.c:1431-1573,
 * one rank, no borders): a header, then one line per level root in index order
 * with index, x, y, z, gval, parent, flux = dh*area, area and the columns of
 * attr_idx's group.  attr_idx must be in the tree's current group. */
dcf_status dcf_tree_export(dcf_ctx *ctx, dcf_tree *tree, int attr_idx, const char *path);
/* Read the primary image of a FITS file as the reference's FITS input does
 * (io.c:624-706, CFITSIO fits_read_pix into float): every pixel BZERO + BSCALE*raw
 * as float, x fastest.  BITPIX 8/16/32/-32/-64, NAXIS 1-3.  dims receives the
 * axis lengths (1 for missing axes), *bitpix the file's BITPIX; out == NULL reads
 * the header only; capacity (in pixels) must cover dims[0]*dims[1]*dims[2]. */
dcf_status dcf_fits_read(const char *path, float *out, uint64_t capacity, uint64_t dims[3], int *bitpix);
/* The same image in its own pixel type, to pass to dcf_tree_build without a float
 * copy (for C2/C3-scale inputs): BITPIX 8 -> DCF_U8, BITPIX 16 with BZERO 32768 ->
 * DCF_U16, BITPIX 32 with BZERO 2147483648 -> DCF_U32, BITPIX -32 -> DCF_F32, all
 * with BSCALE 1 (else DCF_ERR_UNSUPPORTED: use dcf_fits_read).  *dtype receives the
 * dcf_dtype; out == NULL reads the header only; capacity_bytes must cover the data. */
dcf_status dcf_fits_read_raw(const char *path, void *out, uint64_t capacity_bytes, uint64_t dims[3], int *dtype);

/* ---- lambda vectors ---- */
/* Read a "#LambdaVector file..." file: out[0] = 0, out[i] = value_i / imscale.
 * *num_lambdas receives K+1; fails with DCF_ERR_INVALID if capacity < K+1. */
dcf_status dcf_lvec_read(const char *path, double imscale, float *out, int capacity, int *num_lambdas);

#ifdef __cplusplus
}
#endif
#endif
