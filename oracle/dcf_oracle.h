/*
 * CPU restatement of disccofan's component-forest hot path (TEST ORACLE).
 *
 * Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use it as the checker.  The product (libdcf_gb300.so) never
 * links or calls it.  Each function cites the reference file:line it follows.
 *
 * Values are float32 as in the reference (types.h:53-54: `typedef float value`);
 * parents are int64 with -1 for the root (types.h:320 BOTTOM).
 */
#ifndef DCF_ORACLE_H
#define DCF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dco_tree dco_tree;

/* Copy a float image, set dims/pixdim, fix up connectivity (io.c:64-79) and
 * run the extremas + min-tree inversion (preprocessing.c:7-30,77-91).
 * threads = slabs used by the build and chunks used by filters/spectra. */
dco_tree *dco_create(const float *img, uint64_t w, uint64_t h, uint64_t d, int conn, int tree_min,
                     int threads, float pd0, float pd1, float pd2);
void dco_destroy(dco_tree *t);
int dco_connectivity(const dco_tree *t);
float dco_max_gval(const dco_tree *t);

/* Build the tree with the attribute group of attr (flood.c:58-172), or re-flood
 * the attributes of a new group on the existing tree (flood.c:184-219), exactly
 * as loop_operations decides (disccofan.c:148-193). */
int dco_prepare(dco_tree *t, int attr);

int dco_parent(const dco_tree *t, int64_t *out);
int dco_gval(const dco_tree *t, float *out);

/* Attribute (or group area) readout of every level root; NaN elsewhere. */
int dco_node_attr(const dco_tree *t, int attr, int area, double *out);
/* Raw aux records (the reference's AreaData/ExtentData/... layouts), one per pixel. */
int64_t dco_aux(const dco_tree *t, void *out, uint64_t out_bytes);

/* perform_filter_or_extract (operation.c:10-29): rule 0..3, extract, min-tree re-inversion. */
int dco_filter(dco_tree *t, int attr, int rule, double lambda, int extract, float *out);
/* perform_check_operation (operation.c:47-61). */
int dco_check(dco_tree *t, int attr, float *out);
/* 1-D spectrum (pattern.c:27-108, background=1); lv has num_lambdas entries incl. the leading 0. */
int dco_pattern(dco_tree *t, int attr, const float *lv, int n, double *out);
/* 2-D spectrum (pattern.c:110-203) with the attribute-order rule of operation.c:93-100;
 * out[s1 + s2*n1]. attribute 18 = bounding-box elongation on ExtentData. */
int dco_pattern2d(dco_tree *t, int a1, const float *l1, int n1, int a2, const float *l2, int n2,
                  double *out);

/* Symmetric eigenvalues, ascending (stands in for EISPACK rs, eispack.c:12304). */
void dco_sym_eig2(const double m[4], double ev[2]);
void dco_sym_eig3(const double m[9], double ev[3]);

#ifdef __cplusplus
}
#endif
#endif
