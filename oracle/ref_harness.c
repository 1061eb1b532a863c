/*
 * Test-oracle harness around the reference's OWN hot-path C sources.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles the unmodified reference
 * translation units (flood.c, attributes.c, filtering.c, pattern.c, operation.c,
 * queue.c, workspace.c, lambdavec.c, eispack.c, logc.c, checks.c, mpihelper.c,
 * preprocessing.c, csl.c) together with this file and the single-rank mpi.h stub
 * into oracle/_ref/libdcfref.so.  Only tests/ and the CPU-baseline leg of
 * bench.py may load it; the product never does.
 *
 * What this file supplies, and why:
 *  - the globals that the reference defines in disccofan.c:27-49
 *    (g_max_levels, tstruct, start, data_properties, the attribute function
 *    pointers), because disccofan.c itself holds main() and the config/IO layer;
 *  - initialize_attribute_functions (disccofan.c:99-110) and the operation loop
 *    (loop_operations, disccofan.c:137-208) restated for one rank;
 *  - the image writers perform_operation() calls (io.h): here they CAPTURE the
 *    result into a buffer instead of writing files, so operation.c runs unchanged;
 *  - check_connectivity (io.c:64-79) restated, because io.c needs FreeImage/HDF5;
 *  - g_max_levels, which the reference only sets in its ubyte/ushort/uint
 *    preprocessing (preprocessing.c:101,115,129) and which sizes the subtractive
 *    rule's stack arrays (filtering.c:216-217).  It is set to the number of
 *    distinct grey levels + 2, an upper bound on any root path length;
 *  - attribute 18, "bbox elongation" = max(xext,yext)/max(min(xext,yext),1) on
 *    ExtentData, which the reference lacks; it lives here, beside the reference.
 */
#include "types.h"
#include "attributes.h"
#include "flood.h"
#include "filtering.h"
#include "pattern.h"
#include "lambdavec.h"
#include "operation.h"
#include "preprocessing.h"
#include "io.h"
#include <malloc.h>

/* ---- globals the reference defines in disccofan.c ---- */
ulong g_max_levels;
struct tms tstruct;
clock_t start;
DataParams data_properties = {
    .dims_process = {1, 1, 1}, .dims_full = {1, 1, 1}, .pixdim = {1.0, 1.0, 1.0},
    .border = {false, false, false, false, false, false}, .offsets = {0, 0, 0},
    .g_max_gval = 0, .g_min_gval = 0};
f_new_aux_data new_aux_data = NULL;
f_init_aux_data init_aux_data = NULL;
f_delete_aux_data delete_aux_data = NULL;
f_add_to_aux_data add_to_aux_data = NULL;
f_merge_aux_data merge_aux_data = NULL;
f_merge_to_aux_data merge_to_aux_data = NULL;
f_clone_aux_data clone_aux_data = NULL;
f_create_mpi_aux_data create_mpi_aux_data = NULL;
extern int verbosity;

/* ---- harness state ---- */
static Arguments g_args;
static Node *g_tree = NULL;
static int g_prev_attr = -1;
static double g_t_build = 0.0, g_t_op = 0.0;

/* capture buffers filled by the writer stubs */
static void *g_cap = NULL;
static size_t g_cap_bytes = 0;

static void capture(const void *src, size_t bytes)
{
    free(g_cap);
    g_cap = malloc(bytes);
    memcpy(g_cap, src, bytes);
    g_cap_bytes = bytes;
}

/* ---- io.h writers: capture instead of writing files ---- */
void write_no_operation(Arguments *args, value *img, Operation *ope_cur) { (void)args; (void)img; (void)ope_cur; }
void write_filtered(Arguments *args, value *img, Operation *ope_cur)
{ (void)args; (void)ope_cur; capture(img, g_tree->size_init * sizeof(value)); }
void write_check_files(Arguments *args, value *img, Operation *ope_cur)
{ (void)args; (void)ope_cur; capture(img, g_tree->size_init * sizeof(value)); }
void write_pattern_spectra(Arguments *args, Operation *ope_cur, double *spectrum, LambdaVec *lvec)
{ (void)args; (void)ope_cur; capture(spectrum, lvec->num_lambdas * sizeof(double)); }
void write_pattern_spectra2d(Arguments *args, Operation *ope_cur, double *spectrum, LambdaVec *l1, LambdaVec *l2)
{ (void)args; (void)ope_cur; capture(spectrum, (size_t)l1->num_lambdas * l2->num_lambdas * sizeof(double)); }
void write_dmp(Arguments *args, value *out, int num_lambdas, Operation *ope_cur)
{ (void)args; (void)ope_cur; capture(out, (size_t)num_lambdas * g_tree->size_init * sizeof(value)); }
void write_csl(Arguments *args, value *contrast, value *scale, value *luminance, Operation *ope_cur)
{
    (void)args; (void)ope_cur;
    size_t n = g_tree->size_init * sizeof(value);
    free(g_cap);
    g_cap = malloc(3 * n);
    memcpy(g_cap, contrast, n);
    memcpy((char *)g_cap + n, scale, n);
    memcpy((char *)g_cap + 2 * n, luminance, n);
    g_cap_bytes = 3 * n;
}
void write_tree(Arguments *args, Node *tree, Operation *ope_cur) { (void)args; (void)tree; (void)ope_cur; }

/* disccofan.c:99-110 restated */
static void init_attribute_functions(Node *tree, int attr_idx)
{
    tree->size_attr = AttribsArray[attr_idx].size;
    new_aux_data = AttribsArray[attr_idx].new_data;
    init_aux_data = AttribsArray[attr_idx].init_data;
    delete_aux_data = AttribsArray[attr_idx].delete_data;
    add_to_aux_data = AttribsArray[attr_idx].add_to_data;
    merge_aux_data = AttribsArray[attr_idx].merge_data;
    merge_to_aux_data = AttribsArray[attr_idx].merge_to_data;
    clone_aux_data = AttribsArray[attr_idx].clone_data;
    create_mpi_aux_data = AttribsArray[attr_idx].create_mpi_data;
    create_mpi_aux_data();
}

static int cmp_float(const void *a, const void *b)
{
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

void dcfref_free(void)
{
    if (g_tree) {
        free(g_tree->gval);
        free(g_tree->parent);
        free(g_tree->attribute);
        free(g_tree);
        g_tree = NULL;
    }
    free(g_cap);
    g_cap = NULL;
    g_cap_bytes = 0;
    g_prev_attr = -1;
}

/*
 * Load an image (already converted to float, as io.c does for every input type),
 * set data_properties for one rank (no borders, zero offsets) and run the
 * reference's preprocessing (extremas; min-tree inversion, preprocessing.c:77-91).
 * Returns the connectivity after check_connectivity's fix-ups.
 */
int dcfref_load(const float *img, ulong w, ulong h, ulong d, int conn, int tree_min,
                int threads, float pd0, float pd1, float pd2)
{
    dcfref_free();
    verbosity = ERROR;
    /* Allocated-but-unwritten bytes read as zero (M_PERTURB 0xFF fills new
     * allocations with ~0xFF).  perform_operation's output buffer is malloc'ed and
     * the max rule reads entries it has not written yet (filtering.c:177); for real
     * image sizes glibc serves that buffer from fresh zero pages, and this makes the
     * small test images behave the same way. */
    mallopt(M_PERTURB, 0xFF);
    memset(&g_args, 0, sizeof(g_args));
    strcpy(g_args.tree_type, tree_min ? "min" : "max");
    strcpy(g_args.preprocessing, "None");
    g_args.threads = threads > 0 ? threads : 1;
    g_args.pixel_connectivity = conn;
    g_args.save_output = 1;
    g_args.bpp = -32;
    g_args.pixel_dim[0] = pd0; g_args.pixel_dim[1] = pd1; g_args.pixel_dim[2] = pd2;
    omp_set_num_threads(g_args.threads);

    ulong n = w * h * d;
    data_properties.dims_process[0] = data_properties.dims_full[0] = w;
    data_properties.dims_process[1] = data_properties.dims_full[1] = h;
    data_properties.dims_process[2] = data_properties.dims_full[2] = d;
    data_properties.pixdim[0] = pd0; data_properties.pixdim[1] = pd1; data_properties.pixdim[2] = pd2;
    for (int i = 0; i < 6; i++) data_properties.border[i] = false;
    for (int i = 0; i < 3; i++) data_properties.offsets[i] = 0;

    /* io.c:64-79 */
    if (d > 1 && g_args.pixel_connectivity == 4) g_args.pixel_connectivity = 6;
    else if (g_args.pixel_connectivity == 8 && d > 1) g_args.pixel_connectivity = 26;
    else if (g_args.pixel_connectivity == 26 && d == 1) g_args.pixel_connectivity = 8;

    g_tree = malloc(sizeof(Node));
    memset(g_tree, 0, sizeof(Node));
    g_tree->gval = malloc(n * sizeof(value));
    memcpy(g_tree->gval, img, n * sizeof(value));
    g_tree->size_init = g_tree->size_curr = n;

    preprocessing(&g_args, g_tree->gval, n);

    /* number of distinct levels bounds every root path (subtractive rule VLAs) */
    float *tmp = malloc(n * sizeof(float));
    memcpy(tmp, g_tree->gval, n * sizeof(float));
    qsort(tmp, n, sizeof(float), cmp_float);
    ulong distinct = n ? 1 : 0;
    for (ulong i = 1; i < n; i++) distinct += tmp[i] != tmp[i - 1];
    free(tmp);
    g_max_levels = distinct + 2;
    return g_args.pixel_connectivity;
}

/*
 * One entry of the reference's operation list (loop_operations,
 * disccofan.c:137-208, single rank): build on the first call, re-flood the
 * attributes when the group changes, then perform_operation() (operation.c:110).
 * name: filter | extract | check | pattern | pattern2D | dmp | csl | tree.
 * The captured output (image / spectrum / DMP stack) is copied to out when
 * out_bytes matches; returns the captured size in bytes, or -1 on error.
 */
long dcfref_op(const char *name, int attr, int attr2, int rule, double lambda,
               const char *lvec1, double imscale1, const char *lvec2, double imscale2,
               void *out, size_t out_bytes)
{
    if (!g_tree) return -1;
    Operation *op = &g_args.ope_list[0];
    memset(op, 0, sizeof(*op));
    strncpy(op->name, name, 255);
    op->attribute_idx = attr;
    op->attribute_idx_2D = attr2;
    op->decision_idx = rule;
    op->lambda = lambda;
    op->imscale = imscale1 != 0 ? imscale1 : 1.0;
    op->imscale_2D = imscale2 != 0 ? imscale2 : 1.0;
    if (lvec1) strncpy(op->lvec_name, lvec1, 255);
    if (lvec2) strncpy(op->lvec_name_2D, lvec2, 255);
    g_args.num_operations = 1;

    double t0 = omp_get_wtime();
    if (g_prev_attr < 0) {
        init_attribute_functions(g_tree, attr);
        build_tree_with_attributes(&g_args, g_tree);
    } else if (AttribsArray[attr].group != AttribsArray[g_prev_attr].group) {
        free(g_tree->attribute);
        g_tree->attribute = NULL;
        init_attribute_functions(g_tree, attr);
        flood_attributes(g_tree);
    }
    double t1 = omp_get_wtime();
    g_prev_attr = attr;

    Output output = {0};
    free(g_cap);
    g_cap = NULL;
    g_cap_bytes = 0;
    perform_operation(&g_args, g_tree, op, &output);
    double t2 = omp_get_wtime();
    g_t_build = t1 - t0;
    g_t_op = t2 - t1;

    if (out && g_cap && out_bytes == g_cap_bytes) memcpy(out, g_cap, g_cap_bytes);
    return (long)g_cap_bytes;
}

double dcfref_time_build(void) { return g_t_build; }
double dcfref_time_op(void) { return g_t_op; }
ulong dcfref_max_levels(void) { return g_max_levels; }

/* Copy the tree's parent array (canonical after the build's compression). */
int dcfref_parent(int64_t *out)
{
    if (!g_tree || !g_tree->parent) return -1;
    memcpy(out, g_tree->parent, g_tree->size_curr * sizeof(int64_t));
    return 0;
}

/* The grey levels the tree was built on (after min-tree inversion). */
int dcfref_gval(float *out)
{
    if (!g_tree) return -1;
    memcpy(out, g_tree->gval, g_tree->size_curr * sizeof(float));
    return 0;
}

float dcfref_max_gval(void) { return data_properties.g_max_gval; }

/*
 * Attribute readout of every level root (other pixels get NaN): the value
 * AttribsArray[attr].attribute / .area return.  attr must be in the group the
 * current attribute data was built for.
 */
int dcfref_node_attr(int attr, int which_area, double *out)
{
    if (!g_tree || !g_tree->attribute || attr < 0 || attr >= NUMATTR) return -1;
    if (AttribsArray[attr].group != AttribsArray[g_prev_attr].group) return -2;
    double (*fn)(void *) = which_area ? AttribsArray[attr].area : AttribsArray[attr].attribute;
    for (ulong i = 0; i < g_tree->size_curr; i++)
        out[i] = is_levelroot(g_tree, (idx)i) ? fn((char *)g_tree->attribute + i * g_tree->size_attr) : NAN;
    return 0;
}

/* Raw aux record of every pixel (size_attr bytes each). */
long dcfref_aux(void *out, size_t out_bytes)
{
    if (!g_tree || !g_tree->attribute) return -1;
    size_t bytes = g_tree->size_curr * g_tree->size_attr;
    if (out && out_bytes == bytes) memcpy(out, g_tree->attribute, bytes);
    return (long)bytes;
}

/* ---- attribute 18: bounding-box elongation on ExtentData (not a reference attribute) ---- */
double dcfref_bbox_elong(void *rectattr)
{
    double xe = extent_x_attribute(rectattr), ye = extent_y_attribute(rectattr);
    double hi = xe > ye ? xe : ye, lo = xe < ye ? xe : ye;
    return hi / (lo > 1.0 ? lo : 1.0);
}

/*
 * 2-D pattern spectrum with a_1/a_2 allowed to be 18 (bbox elongation), through
 * the reference's own tree_pattern_spectrum2d (pattern.c:110).  Same argument
 * rules as perform_pattern_spectrum (operation.c:93-100): when a2 == 0 the second
 * attribute is the first attribute's group area.
 */
int dcfref_pattern2d_ext(int a1, const char *lvec1, double imscale1, int a2, const char *lvec2,
                         double imscale2, double *out)
{
    if (!g_tree || !g_tree->attribute) return -1;
    int group = AttribsArray[g_prev_attr].group;
    if (group != 1) return -2;
    LambdaVec *l1 = lambda_vector_read((char *)lvec1, imscale1);
    LambdaVec *l2 = lambda_vector_read((char *)lvec2, imscale2);
    if (!l1 || !l2) return -3;
    double (*f1)(void *) = a1 == 18 ? dcfref_bbox_elong : AttribsArray[a1].attribute;
    double (*f2)(void *) = a2 == 18 ? dcfref_bbox_elong
                         : (a2 == 0 ? AttribsArray[1].area : AttribsArray[a2].attribute);
    double (*fa)(void *) = AttribsArray[1].area;
    memset(out, 0, (size_t)l1->num_lambdas * l2->num_lambdas * sizeof(double));
    tree_pattern_spectrum2d(g_tree, g_tree->size_init, l1, l2, g_tree->area_copy, g_tree->gval_par,
                            out, 1, fa, f1, f2);
    lambda_vector_delete(l1);
    lambda_vector_delete(l2);
    return 0;
}
