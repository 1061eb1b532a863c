/*
 * dcf_reftypes.h -- the reference's data layouts that its hot-path functions take,
 * declared byte for byte so that code built against them links with code built
 * against the reference's own src/headers/types.h.
 *
 * Used by the link-compatible replacement of the reference's hot-path functions
 * (disccofan_gb300/csrc/dcf_refshim.c, libdcf_refshim.so) when it is compiled
 * without the reference checkout, and by programs that call that replacement.
 * The layouts mirror, field for field and in order:
 *   LambdaVec           src/headers/types.h:64-67
 *   Operation           src/headers/types.h:70-82
 *   DataParams          src/headers/types.h:84-92
 *   Arguments           src/headers/types.h:96-126
 *   AuxDataStore        src/headers/types.h:137-143
 *   Node                src/headers/types.h:147-159
 *   AttribStruct        src/headers/types.h:297-312
 * with the reference's scalar types (types.h:37-54: value = float, idx = int64_t,
 * ulong = uint64_t) and constants (NUMATTR, BOTTOM, MAX_OPERATION_SIZE).  A CPU
 * test compares every field offset and size with the reference's header.
 *
 * The globals a caller of the replacement provides, as the reference's
 * disccofan.c and attributes.c do: AttribsArray (the attribute table, used to map
 * the function pointers the reference passes back to attribute indices),
 * data_properties (image dimensions and pixel size) and init_aux_data (the
 * attribute group currently selected, disccofan.c:99-110).
 */
#ifndef DCF_REFTYPES_H
#define DCF_REFTYPES_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint8_t ubyte;
typedef uint16_t ushort;
typedef uint32_t uint;
typedef uint64_t ulong;
typedef int64_t idx;
typedef float value;

#define MAX_OPERATION_SIZE 10
#define NUMATTR 18
#define BOTTOM (-1)

typedef struct _LambdaVec {
    uint num_lambdas;
    float *lambdas;
} LambdaVec;

typedef struct _Operation {
    char name[256];
    char lvec_name[256];
    char lvec_name_2D[256];
    int attribute_idx;
    int attribute_idx_2D;
    int decision_idx;
    double lambda;
    double imscale;
    double imscale_2D;
    LambdaVec *lvec1;
    LambdaVec *lvec2;
} Operation;

typedef struct _DataParams {
    ulong dims_process[3];
    ulong dims_full[3];
    float pixdim[3];
    bool border[6];
    long offsets[3];
    value g_max_gval;
    value g_min_gval;
} DataParams;

typedef struct _Arguments {
    int interactive;
    char folder_run[256], config_file[256], input_name[256], output_name[256];
    char input_prefix[256], output_prefix[256], input_type[256], output_type[256];
    char hdf5_dataset[256], image_options[256], tree_type[256], input_file_style[256];
    char output_file_style[256], verbosity[256], preprocessing[256];
    int tile_overlap;
    int mpi_grid[3];
    float pixel_dim[3];
    int threads;
    int bpp;
    int pixel_connectivity;
    int include_background;
    int save_output;
    int save_tree;
    int num_operations;
    int image_stats;
    Operation ope_list[MAX_OPERATION_SIZE];
} Arguments;

typedef struct _AuxDataStore {
    void *data;
    size_t size_item;
    ulong size_alloc;
    ulong item_curr;
} AuxDataStore;

typedef struct _Node {
    idx *parent;
    idx *border_idx;
    void *attribute;
    double *area_copy;
    value *gval;
    value *gval_par;
    ulong size_init;
    ulong size_curr;
    ulong size_attr;
    ulong offsets[3];
    bool border[6];
} Node;

typedef struct _AttribStruct {
    const char *name;
    const char *short_name;
    ulong size;
    uint group;
    void *(*new_data)(AuxDataStore *);
    void (*init_data)(void *, bool, ulong, ulong, ulong, value);
    void (*delete_data)(void *);
    void (*add_to_data)(void *, void *);
    void (*merge_data)(void *, void *);
    void (*merge_to_data)(AuxDataStore *, void **, void *, void *);
    void (*clone_data)(AuxDataStore *, void **, void *);
    void (*create_mpi_data)(void);
    double (*area)(void *);
    double (*attribute)(void *);
} AttribStruct;

typedef void (*f_init_aux_data)(void *, bool, ulong, ulong, ulong, value);

extern AttribStruct AttribsArray[NUMATTR];
extern DataParams data_properties;
extern f_init_aux_data init_aux_data;

/* The replaced functions, with the reference's signatures (flood.h:5,7,33;
 * filtering.h:6-7; pattern.h:4,6). */
void build_tree_with_attributes(Arguments *args, Node *local_tree);
void flood_attributes(Node *local_tree);
idx get_levelroot(Node *tree, idx x);
void tree_filtering(Node *tree, value *out, ulong size_tile, int decision_choice, int attrib_choice, double lambda);
void tree_attribute_check(Node *tree, value *out, ulong lwb, ulong upb, double (*attribute)(void *));
void tree_pattern_spectrum(Node *tree, ulong size, LambdaVec *lvec, double *copy_attr, value *gvals_par,
                           double *spectrum, bool background, double (*area)(void *), double (*attribute)(void *));
void tree_pattern_spectrum2d(Node *tree, ulong size, LambdaVec *lvec_attr1, LambdaVec *lvec_attr2, double *copy_attr,
                             value *gvals_par, double *spectrum, int background, double (*area)(void *),
                             double (*attribute1)(void *), double (*attribute2)(void *));

/* No reference counterpart: frees the device tree the replacement keeps for this
 * Node (call it where the reference's free_tree, disccofan.c:64-74, frees one). */
void dcf_refshim_release(Node *tree);

#ifdef __cplusplus
}
#endif
#endif
