/*
 * Calls the reference-signature replacement (libdcf_refshim.so) the way the
 * reference's operation.c and disccofan.c call flood.c, filtering.c and pattern.c,
 * on one 2-D float image, and writes every result as a raw binary file.
 *
 *   refshim_driver <image.f32> <width> <height> <connectivity> <out_dir>
 *
 * This program stands in for the reference's attributes.c and disccofan.c: it owns
 * the globals the replacement reads (AttribsArray, data_properties, init_aux_data).
 * Its attribute table holds functions that are never called -- the replacement
 * only compares their addresses -- laid out like the reference's
 * (attributes.c:1224-1248): entry i's `attribute` is attribute i, and every entry of
 * a group shares the group's `area` and `init_data`, with entry 0's area readout
 * being its attribute.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "dcf_reftypes.h"

#define NEVER(name) \
    static double name(void *p) { (void)p; abort(); }
NEVER(attr0) NEVER(attr1) NEVER(attr2) NEVER(attr3) NEVER(attr4) NEVER(attr5) NEVER(attr6) NEVER(attr7) NEVER(attr8)
NEVER(attr9) NEVER(attr10) NEVER(attr11) NEVER(attr12) NEVER(attr13) NEVER(attr14) NEVER(attr15) NEVER(attr16)
NEVER(attr17) NEVER(area1) NEVER(area2) NEVER(area3) NEVER(area4)
#define INIT(name) \
    static void name(void *a, bool b, ulong c, ulong d, ulong e, value f) { (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; abort(); }
INIT(init0) INIT(init1) INIT(init2) INIT(init3) INIT(init4)

static double (*const ATTR[NUMATTR])(void *) = {attr0, attr1, attr2, attr3, attr4, attr5, attr6, attr7, attr8,
                                                attr9, attr10, attr11, attr12, attr13, attr14, attr15, attr16, attr17};
static const int GROUP[NUMATTR] = {0, 1, 1, 1, 1, 1, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4};

AttribStruct AttribsArray[NUMATTR];
DataParams data_properties;
f_init_aux_data init_aux_data;

static void fill_table(void)
{
    double (*const area[5])(void *) = {attr0, area1, area2, area3, area4};
    const f_init_aux_data init[5] = {init0, init1, init2, init3, init4};
    for (int i = 0; i < NUMATTR; i++) {
        AttribsArray[i].attribute = ATTR[i];
        AttribsArray[i].area = area[GROUP[i]];
        AttribsArray[i].init_data = init[GROUP[i]];
        AttribsArray[i].group = (uint)GROUP[i];
    }
}

static void put(const char *dir, const char *name, const void *data, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f || fwrite(data, 1, bytes, f) != bytes) {
        fprintf(stderr, "cannot write %s\n", path);
        exit(2);
    }
    fclose(f);
}

/* initialize_attribute_functions (disccofan.c:99-110), as far as the replacement reads it */
static void select_attribute(Node *tree, int a)
{
    init_aux_data = AttribsArray[a].init_data;
    tree->size_attr = 0;
}

int main(int argc, char **argv)
{
    if (argc != 6) {
        fprintf(stderr, "usage: %s image.f32 width height connectivity out_dir\n", argv[0]);
        return 2;
    }
    const ulong W = strtoul(argv[2], NULL, 10), H = strtoul(argv[3], NULL, 10), N = W * H;
    const char *out_dir = argv[5];
    fill_table();

    Node tree;
    memset(&tree, 0, sizeof(tree));
    tree.gval = (value *)malloc(N * sizeof(value));
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(tree.gval, sizeof(value), N, f) != N) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    fclose(f);
    tree.size_init = tree.size_curr = N;
    data_properties.dims_process[0] = W;
    data_properties.dims_process[1] = H;
    data_properties.dims_process[2] = 1;
    for (int i = 0; i < 3; i++) data_properties.pixdim[i] = 1.0f;

    static Arguments args;  /* large: kept off the stack */
    args.pixel_connectivity = atoi(argv[4]);
    args.threads = 1;

    value *out = (value *)malloc(N * sizeof(value));
    idx *lr = (idx *)malloc(N * sizeof(idx));

    /* ("filter", 0, 200) on the area group */
    select_attribute(&tree, 0);
    build_tree_with_attributes(&args, &tree);
    put(out_dir, "parent.i64", tree.parent, N * sizeof(idx));
    for (ulong x = 0; x < N; x++) lr[x] = get_levelroot(&tree, (idx)x);
    put(out_dir, "levelroot.i64", lr, N * sizeof(idx));
    tree_filtering(&tree, out, tree.size_init, 0, 0, 200.0);
    put(out_dir, "filter_area_200.f32", out, N * sizeof(value));
    /* ("check", 0), once per thread range as perform_check_operation does */
    memset(out, 0, N * sizeof(value));
    tree_attribute_check(&tree, out, 0, N / 3, AttribsArray[0].attribute);
    tree_attribute_check(&tree, out, N / 3, N, AttribsArray[0].attribute);
    put(out_dir, "check_area.f32", out, N * sizeof(value));
    /* ("pattern", 0, lvec): bins as lambda_vector_read builds them, leading 0 */
    float l_area[5] = {0.0f, 2.0f, 10.0f, 50.0f, 200.0f};
    LambdaVec lv_area = {5, l_area};
    double spec1[5] = {0};
    tree_pattern_spectrum(&tree, tree.size_init, &lv_area, tree.area_copy, tree.gval_par, spec1, 1,
                          AttribsArray[0].area, AttribsArray[0].attribute);
    put(out_dir, "pattern_area.f64", spec1, sizeof(spec1));

    /* a new group: the reference re-floods the attributes (disccofan.c:179-193) */
    select_attribute(&tree, 14);
    flood_attributes(&tree);
    tree_filtering(&tree, out, tree.size_init, 0, 17, 0.2);
    put(out_dir, "filter_ncomp_0.2.f32", out, N * sizeof(value));
    tree_attribute_check(&tree, out, 0, N, AttribsArray[17].attribute);
    put(out_dir, "check_ncomp.f32", out, N * sizeof(value));
    /* ("pattern2D", 14, lvec, 0, lvec): the second attribute is the group's area
     * readout, AttribsArray[14].area (operation.c:96-97) */
    float l_elong[4] = {0.0f, 1.5f, 2.0f, 4.0f};
    LambdaVec lv_elong = {4, l_elong};
    double spec2[4 * 5] = {0};
    tree_pattern_spectrum2d(&tree, tree.size_init, &lv_elong, &lv_area, tree.area_copy, tree.gval_par, spec2, 1,
                            AttribsArray[14].area, AttribsArray[14].attribute, AttribsArray[14].area);
    put(out_dir, "pattern2d_14_0.f64", spec2, sizeof(spec2));

    dcf_refshim_release(&tree);
    free(tree.parent);
    free(tree.gval);
    free(out);
    free(lr);
    printf("refshim driver ok\n");
    return 0;
}
