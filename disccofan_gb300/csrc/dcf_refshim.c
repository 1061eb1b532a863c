/*
 * dcf_refshim.c -- link-compatible replacement of the reference's hot-path
 * functions on top of the C ABI (libdcf_gb300.so).  Built as libdcf_refshim.so.
 *
 * A program written against the reference (its operation.c / disccofan.c) links
 * this library instead of flood.c's, filtering.c's and pattern.c's definitions of
 *
 *   build_tree_with_attributes   src/headers/flood.h:5      src/sources/flood.c:175
 *   flood_attributes             src/headers/flood.h:7      src/sources/flood.c:184
 *   get_levelroot                src/headers/flood.h:33     src/sources/flood.c:693
 *   tree_filtering               src/headers/filtering.h:6  src/sources/filtering.c:18
 *   tree_attribute_check         src/headers/filtering.h:7  src/sources/filtering.c:47
 *   tree_pattern_spectrum        src/headers/pattern.h:4    src/sources/pattern.c:27
 *   tree_pattern_spectrum2d      src/headers/pattern.h:6    src/sources/pattern.c:110
 *
 * and keeps its call sites unchanged.  Compiled with -DDCF_REFSHIM_REFERENCE_HEADERS
 * and the reference's src/headers on the include path, it takes the reference's
 * own types.h and prototypes (so the compiler checks every signature against
 * them) and reports failures through the reference's error() and MPI_Abort;
 * otherwise it takes include/dcf_reftypes.h, the same layouts declared here, and
 * reports through stderr and abort().
 *
 * What the reference keeps in globals the shim reads from the same globals:
 *   - the image: Node.gval (float, x fastest; a min-tree image is already inverted
 *     by preprocessing.c:84-91), data_properties.dims_process and .pixdim;
 *   - the connectivity: Arguments.pixel_connectivity (io.c:64-79's fix-ups are
 *     applied by dcf_tree_build);
 *   - the attribute group: init_aux_data, set by initialize_attribute_functions
 *     (disccofan.c:99-110) to AttribsArray[i].init_data of the selected attribute;
 *   - attributes passed as function pointers: AttribsArray[i].attribute is
 *     attribute i, and any AttribsArray[i].area is the area (attribute 0) -- the
 *     reference passes a group's area readout as the second attribute of
 *     "pattern2D a, 0" (operation.c:96-97).
 *
 * The tree itself stays on the device (one dcf_tree per Node).  After a build,
 * Node.parent holds the canonical parent array (malloc'ed like flood.c:93-94, freed
 * by the caller's free_tree), so code that walks parents or calls get_levelroot
 * keeps working.  Node.attribute stays NULL: attribute readouts go through the
 * functions above.  dcf_refshim_release(node) frees a Node's device tree (a
 * maintainer calls it from free_tree, disccofan.c:64-74).
 *
 * Every reference caller passes background = 1 to the spectra (operation.c:82,
 * 96-99), which is what the library computes (the root's dh is its level); a call
 * with background = 0 is refused.  The spectra accumulate into the caller's array
 * (+=), as pattern.c:98-105 does.  The reference's errors abort (check_alloc,
 * checks.c:4-24); so do the shim's.
 */
#ifdef DCF_REFSHIM_REFERENCE_HEADERS
#include "types.h"
#include "flood.h"
#include "filtering.h"
#include "pattern.h"
#else
#include <stdio.h>
#include <stdlib.h>
#include "dcf_reftypes.h"
#endif

#include <pthread.h>
#include <string.h>

#include "dcf.h"

#ifdef DCF_REFSHIM_REFERENCE_HEADERS
void dcf_refshim_release(Node *tree);
#endif

static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;
static dcf_ctx *g_ctx;

/* Node -> device tree; a handful of live trees at most (the reference keeps one) */
typedef struct Binding {
    Node *node;
    dcf_tree *tree;
    int check_attr;   /* attribute of the cached check image, -1: none */
    value *check;     /* tree_attribute_check is called once per OpenMP thread */
    struct Binding *next;
} Binding;
static Binding *g_bindings;

static void fail(const char *what, dcf_status s)
{
    const char *detail = g_ctx ? dcf_ctx_last_error(g_ctx) : "";
#ifdef DCF_REFSHIM_REFERENCE_HEADERS
    error("dcf: %s: %s (%s)", what, dcf_status_string(s), detail);
    MPI_Abort(MPI_COMM_WORLD, 1);
#else
    fprintf(stderr, "dcf: %s: %s (%s)\n", what, dcf_status_string(s), detail);
    abort();
#endif
}

static void ok(dcf_status s, const char *what)
{
    if (s != DCF_OK) fail(what, s);
}

static Binding *binding(Node *tree, int create)
{
    for (Binding *b = g_bindings; b; b = b->next)
        if (b->node == tree) return b;
    if (!create) return NULL;
    Binding *b = (Binding *)calloc(1, sizeof(Binding));
    if (!b) fail("binding", DCF_ERR_NOMEM);
    b->node = tree;
    b->check_attr = -1;
    b->next = g_bindings;
    g_bindings = b;
    return b;
}

static dcf_tree *tree_of(Node *tree, const char *what)
{
    Binding *b = binding(tree, 0);
    if (!b || !b->tree) fail(what, DCF_ERR_STATE);
    return b->tree;
}

static void drop_check(Binding *b)
{
    free(b->check);
    b->check = NULL;
    b->check_attr = -1;
}

/* the attribute index of a readout the reference passes as a function pointer */
static int attr_of(double (*fn)(void *), const char *what)
{
    for (int i = 0; i < NUMATTR; i++)
        if (AttribsArray[i].attribute == fn) return i;
    for (int i = 0; i < NUMATTR; i++)
        if (AttribsArray[i].area == fn) return 0;
    fail(what, DCF_ERR_INVALID);
    return -1;
}

/* the attribute the reference's initialize_attribute_functions selected (any
 * member of its group: only the group matters for the records) */
static int current_attr(void)
{
    for (int i = 0; i < NUMATTR; i++)
        if (AttribsArray[i].init_data == init_aux_data) return i;
    fail("no attribute group selected (init_aux_data)", DCF_ERR_STATE);
    return -1;
}

void build_tree_with_attributes(Arguments *args, Node *local_tree)
{
    pthread_mutex_lock(&g_mu);
    if (!g_ctx) ok(dcf_ctx_create(0, NULL, &g_ctx), "dcf_ctx_create");
    Binding *b = binding(local_tree, 1);
    if (b->tree) dcf_tree_destroy(b->tree);
    b->tree = NULL;
    drop_check(b);
    dcf_image img;
    memset(&img, 0, sizeof(img));
    img.data = local_tree->gval;
    img.dtype = DCF_F32;
    img.on_device = 0;
    for (int i = 0; i < 3; i++) {
        img.dims[i] = data_properties.dims_process[i];
        img.pixdim[i] = data_properties.pixdim[i];
    }
    img.connectivity = args->pixel_connectivity;
    img.tree_type = DCF_MAX_TREE;
    ok(dcf_tree_build(g_ctx, &img, current_attr(), &b->tree), "build_tree_with_attributes");
    const ulong n = img.dims[0] * img.dims[1] * (img.dims[2] ? img.dims[2] : 1);
    local_tree->size_init = local_tree->size_curr = n;
    free(local_tree->parent);
    local_tree->parent = (idx *)malloc(n * sizeof(idx));
    if (!local_tree->parent) fail("build_tree_with_attributes: parent", DCF_ERR_NOMEM);
    ok(dcf_tree_parent(g_ctx, b->tree, (int64_t *)local_tree->parent, 0), "build_tree_with_attributes: parent");
    pthread_mutex_unlock(&g_mu);
}

void flood_attributes(Node *local_tree)
{
    pthread_mutex_lock(&g_mu);
    Binding *b = binding(local_tree, 0);
    dcf_tree *t = tree_of(local_tree, "flood_attributes");
    drop_check(b);
    ok(dcf_tree_set_attribute(g_ctx, t, current_attr()), "flood_attributes");
    pthread_mutex_unlock(&g_mu);
}

/* Node.parent is in canonical form: a pixel that is not a level root points to
 * its level root, which has the same grey level */
idx get_levelroot(Node *tree, idx x)
{
    const idx p = tree->parent[x];
    return (p != BOTTOM && tree->gval[p] == tree->gval[x]) ? p : x;
}

void tree_filtering(Node *tree, value *out, ulong size_tile, int decision_choice, int attrib_choice, double lambda)
{
    pthread_mutex_lock(&g_mu);
    dcf_tree *t = tree_of(tree, "tree_filtering");
    uint64_t n = 0;
    ok(dcf_tree_info(t, &n, NULL, NULL, NULL), "tree_filtering");
    if (size_tile != n) fail("tree_filtering: size_tile is not the tree's pixel count", DCF_ERR_INVALID);
    ok(dcf_filter(g_ctx, t, attrib_choice, decision_choice, lambda, 0, out, 0), "tree_filtering");
    pthread_mutex_unlock(&g_mu);
}

/* Called once per OpenMP thread with its own [lwb, upb) (operation.c:47-61): the
 * check image is computed by the first call and copied range by range. */
void tree_attribute_check(Node *tree, value *out, ulong lwb, ulong upb, double (*attribute)(void *))
{
    pthread_mutex_lock(&g_mu);
    Binding *b = binding(tree, 0);
    dcf_tree *t = tree_of(tree, "tree_attribute_check");
    const int a = attr_of(attribute, "tree_attribute_check: unknown attribute function");
    uint64_t n = 0;
    ok(dcf_tree_info(t, &n, NULL, NULL, NULL), "tree_attribute_check");
    if (upb > n || lwb > upb) fail("tree_attribute_check: range", DCF_ERR_INVALID);
    if (b->check_attr != a) {
        drop_check(b);
        b->check = (value *)malloc(n * sizeof(value));
        if (!b->check) fail("tree_attribute_check", DCF_ERR_NOMEM);
        ok(dcf_attribute_check(g_ctx, t, a, b->check, 0), "tree_attribute_check");
        b->check_attr = a;
    }
    memcpy(out + lwb, b->check + lwb, (upb - lwb) * sizeof(value));
    pthread_mutex_unlock(&g_mu);
}

void tree_pattern_spectrum(Node *tree, ulong size, LambdaVec *lvec, double *copy_attr, value *gvals_par,
                           double *spectrum, bool background, double (*area)(void *), double (*attribute)(void *))
{
    (void)size;
    (void)copy_attr;  /* the multi-rank corrections (pattern.c:46-79) have no counterpart: one device tree */
    (void)gvals_par;
    (void)area;       /* the group's area, which the library bins with */
    pthread_mutex_lock(&g_mu);
    dcf_tree *t = tree_of(tree, "tree_pattern_spectrum");
    if (!background) fail("tree_pattern_spectrum: background = 0 is not supported", DCF_ERR_UNSUPPORTED);
    const int a = attr_of(attribute, "tree_pattern_spectrum: unknown attribute function");
    ok(dcf_pattern_spectrum(g_ctx, t, a, lvec->lambdas, (int)lvec->num_lambdas, spectrum, 0), "tree_pattern_spectrum");
    pthread_mutex_unlock(&g_mu);
}

void tree_pattern_spectrum2d(Node *tree, ulong size, LambdaVec *lvec_attr1, LambdaVec *lvec_attr2, double *copy_attr,
                             value *gvals_par, double *spectrum, int background, double (*area)(void *),
                             double (*attribute1)(void *), double (*attribute2)(void *))
{
    (void)size;
    (void)copy_attr;
    (void)gvals_par;
    (void)area;
    pthread_mutex_lock(&g_mu);
    dcf_tree *t = tree_of(tree, "tree_pattern_spectrum2d");
    if (!background) fail("tree_pattern_spectrum2d: background = 0 is not supported", DCF_ERR_UNSUPPORTED);
    const int a1 = attr_of(attribute1, "tree_pattern_spectrum2d: unknown attribute function");
    const int a2 = attr_of(attribute2, "tree_pattern_spectrum2d: unknown attribute function");
    ok(dcf_pattern_spectrum2d(g_ctx, t, a1, lvec_attr1->lambdas, (int)lvec_attr1->num_lambdas, a2,
                              lvec_attr2->lambdas, (int)lvec_attr2->num_lambdas, spectrum, 0),
       "tree_pattern_spectrum2d");
    pthread_mutex_unlock(&g_mu);
}

void dcf_refshim_release(Node *tree)
{
    pthread_mutex_lock(&g_mu);
    for (Binding **pb = &g_bindings; *pb; pb = &(*pb)->next) {
        Binding *b = *pb;
        if (b->node != tree) continue;
        if (b->tree) dcf_tree_destroy(b->tree);
        drop_check(b);
        *pb = b->next;
        free(b);
        break;
    }
    pthread_mutex_unlock(&g_mu);
}
