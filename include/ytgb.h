/*
 * ytgb.h -- C ABI of the GB300 ray-casting sampler library (libytgb.so).
 *
 * The library replaces the native layer under yt's ImageSampler call surface
 * (yt/utilities/lib/image_samplers.pyx): the per-brick Cython loop
 * cast_through_kdtree + walk_volume + sampler callbacks becomes one CUDA
 * launch over every brick of a view.  Every entry point is plain C: pointers,
 * sizes, an int status (0 = ok, < 0 = error, message in ytgb_last_error()).
 * Device pointers are owned by the caller (e.g. torch tensors); the library
 * allocates no device memory.  `stream` is a cudaStream_t passed as void*.
 */
#ifndef YTGB_H
#define YTGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YTGB_ABI_VERSION 4

#define YTGB_OK 0
#define YTGB_ERR_INVALID (-1)   /* bad argument, detected on the host */
#define YTGB_ERR_CUDA (-2)      /* a CUDA runtime call failed */
#define YTGB_ERR_DEVICE (-3)    /* a device-side guard tripped (see error word) */

/* sampler kinds: VolumeRenderSampler (image_samplers.pyx:405-487),
 * ProjectionSampler (:327-343), InterpolatedProjectionSampler (:346-403),
 * the MIP sampler (ProjectionSampler with max; no reference counterpart) and
 * LightSourceRenderSampler (:496-590). */
#define YTGB_VOLUME_RENDER 0
#define YTGB_PROJECTION 1
#define YTGB_INTERPOLATED_PROJECTION 2
#define YTGB_MIP 3
#define YTGB_LIGHT_SOURCE 4

/* ray generation: generate_vector_info_plane_parallel (lenses.pyx:179-192);
 * generate_vector_info_null, i.e. per-pixel arrays (lenses.pyx:196-207); or
 * the per-pixel rays of PerspectiveLens._get_sampler_params (lens.py:166-234)
 * computed on the device from the camera instead of read from arrays */
#define YTGB_LENS_PLANE_PARALLEL 0
#define YTGB_LENS_PER_PIXEL 1
#define YTGB_LENS_PERSPECTIVE 2

/* pixel culling: calculate_extent_plane_parallel / _perspective / _null
 * (lenses.pyx:22-55, :60-161, :169-175) */
#define YTGB_EXTENT_PLANE_PARALLEL 0
#define YTGB_EXTENT_PERSPECTIVE 1
#define YTGB_EXTENT_NULL 2

/* render flags */
#define YTGB_FLAG_NO_COMPENSATION 1u   /* plain FP32 accumulation (precision study) */
#define YTGB_FLAG_TILE_SHIFT 8         /* bits 8..11: tile shape 0 = 8x16, 1 = 16x8, 2 = 4x32 pixels */

/* One brick: the fields of yt's VolumeContainer (volume_container.pxd:13-33,
 * filled by PartitionedGrid.__cinit__, partitioned_grid.pyx:28-63), plus
 * per-brick constants of walk_volume precomputed on the host with the same
 * float64 operations.  The brick's field f occupies
 * data[data_offset + f*field_stride ...] in the float32 arena: (dims+1)^3
 * vertex values for vertex-centred samplers, dims^3 cell values for
 * ProjectionSampler / MIP, C order. */
typedef struct ytgb_brick {
    double left_edge[3];
    double right_edge[3];
    double dds[3];        /* (right_edge - left_edge) / dims */
    double idds[3];       /* 1 / dds */
    double snap[3];       /* 1e-10 * dds: face snapping tolerance (grid_traversal.pyx:67-74) */
    int32_t dims[3];
    int32_t n_fields;
    int64_t data_offset;  /* float index of field 0 */
    int64_t field_stride; /* floats between consecutive fields */
    int64_t mask_offset;  /* byte index into the mask arena; -1 = all ones */
    int64_t bounds_offset;/* double index of the cell-boundary table (k*dds + le,
                           * k = 0..dims, per axis: grid_traversal.pyx:106-108) */
    float lef[3], ref[3], iddsf[3];  /* float32 copies for conservative pre-tests */
    int32_t pad[5];
} ytgb_brick;

/* The device layout of n bricks: their descriptors (the VolumeContainer
 * fields of PartitionedGrid.__cinit__, partitioned_grid.pyx:47-63, in the
 * same float64 operations, plus arena offsets: each field sizes_max[k]
 * floats rounded up to a multiple of 4, the bricks' fields back to back;
 * mask_offset -1) and the cell-boundary tables k*dds + le, k = 0..dims,
 * per brick and axis, into bounds (sum of dims+1 entries).  *arena_len is
 * the arena's length in floats. */
int ytgb_brick_layout(int64_t n, const int64_t *dims, const double *le, const double *re, const int64_t *n_fields,
                      const int64_t *sizes_max, ytgb_brick *desc, double *bounds, int64_t bounds_len,
                      int64_t *arena_len);

/* One view: the ray-generation and culling fields of ImageSampler
 * (image_samplers.pxd:38-70, set in ImageSampler.__init__ :59-131). */
typedef struct ytgb_view {
    int32_t nx, ny;           /* image.shape[0], image.shape[1] (nv) */
    int32_t lens;             /* YTGB_LENS_* */
    int32_t extent;           /* YTGB_EXTENT_* */
    double vp_pos[12];        /* plane-parallel: inv_mat.ravel('F') + back_center;
                               * perspective: position, east, north, normal */
    double vp_dir[3];         /* plane-parallel: normal * width[2]; perspective: width */
    double center[3];
    double bounds[4];
    double x_vec[3];
    double y_vec[3];
    double width[3];
    double camera_data[15];   /* position, width, east, north, normal */
    double pdx, pdy;          /* (bounds[1]-bounds[0])/nx, (bounds[3]-bounds[2])/ny */
    double ray_scale;         /* perspective: max_length / width[2] (lens.py:204-211) */
    /* derived by the library from the fields above before each launch and in
     * ytgb_batch_plan (callers need not set them): the perspective lens's
     * linspace steps 1/(nx-1), 1/(ny-1) (0 for one pixel) and normal * width[2] */
    double lin_step[2];
    double normal_w2[3];
    const double *px_pos;     /* device (nx,ny,3) for YTGB_LENS_PER_PIXEL, else NULL */
    const double *px_dir;     /* device (nx,ny,3) for YTGB_LENS_PER_PIXEL, else NULL */
} ytgb_view;

/* Transfer function, packed for the device by ytgb_tf_pack from yt's
 * FieldInterpolationTable set (field_interpolation_tables.pxd:27-61 and the
 * VolumeRenderAccumulator of image_samplers.pyx:45-55). */
#define YTGB_TF_MAX_TABLES 6
#define YTGB_TF_MAX_BINS 4096
typedef struct ytgb_tf {
    int32_t n_fits;
    int32_t grey_opacity;
    int32_t nbins_max;
    int32_t ctf_fast;                  /* 1: ColorTransferFunction layout */
    int32_t field_table_ids[6];
    int32_t field_id[6];
    int32_t weight_field_id[6];
    int32_t weight_table_id[6];
    int32_t nbins[6];
    float lo_excl[6];   /* largest float <= bounds[0]: v <= lo_excl -> 0 */
    float hi_excl[6];   /* smallest float >= bounds[1]: v >= hi_excl -> 0 */
    float b0[6];        /* bounds[0] as float, for the bin index */
    float idbin[6];     /* 1/dbin as float, for the bin index */
    double bound64[6][2]; /* the bounds as given: a sample whose float32 value lies
                           * within its rounding error of a bound (or of 0) is
                           * decided in float64, as FIT_get_value does */
    /* table floats follow in a separate buffer: for table t, bin b:
     * tab[(t*nbins_max + b)*4 + {0,1,2,3}] = {y, dy, d0_hi, d0_lo} */
} ytgb_tf;

/* Arguments of one render: cast_through_kdtree (image_samplers.pyx:146-197)
 * for every brick of `order`, in that order, in one launch. */
typedef struct ytgb_render_args {
    int32_t kind;              /* YTGB_VOLUME_RENDER ... YTGB_LIGHT_SOURCE */
    int32_t n_samples;         /* samples per cell (VR / interpolated projection) */
    int32_t n_order;           /* number of entries in order / rects */
    uint32_t flags;            /* YTGB_FLAG_* */
    ytgb_view view;
    const ytgb_brick *bricks;  /* device */
    const int32_t *order;      /* device: brick indices in viewpoint order */
    const int32_t *rects;      /* device: 4 per order entry, from ytgb_brick_rects */
    const float *data;         /* device float32 arena */
    const uint8_t *masks;      /* device mask arena, or NULL when all are -1 */
    const double *bounds;      /* device cell-boundary tables (see ytgb_brick) */
    ytgb_tf tf;                /* by value, from ytgb_tf_pack (VR and light source) */
    const float *tf_tables;    /* device, VR and light source */
    double *image;             /* device (nx,ny,4) float64, updated in place (or host
                                * memory, where the device reads and writes pageable host
                                * memory: see ytgb_device_reads_host) */
    const double *zbuffer;     /* device (nx,ny) float64, or NULL (all ones); host memory
                                * as for image */
    unsigned long long *counters; /* device [4]: cell visits, ray-brick walks, rays, cells
                                  * outside their brick (skipped); or NULL */
    int32_t *error;            /* device error word (0 = ok), or NULL */
    const float *data_lo;      /* device: data - (float)data for every arena value, or
                                * NULL (taken as 0): the light-source gradient's
                                * differences, and the range decisions below */
    /* LightSourceRenderSampler only (image_samplers.pyx:496-590) */
    float light_dir[3];        /* normalised light direction */
    float light_rgba[4];
    /* Volume rendering and light source with data_lo: M * 2^-24, M >= every
     * |value| of the arena.  A sample whose float32 value is 0 or lies within
     * range_eps * (96 + 16 * (dims0 + dims1 + dims2 + 3)) of a transfer-function
     * bound (its float32 error bound, twice over) is decided as FIT_get_value
     * decides it (field_interpolation_tables.pxd:66-80): from yt's float64
     * value, recomputed from data + data_lo.  0: float32 decisions only. */
    float range_eps;
} ytgb_render_args;

/* One view of a multi-view batch (device memory), as filled by
 * ytgb_batch_plan: the view's render arguments plus its place in the batch's
 * tile numbering. */
typedef struct ytgb_batch_entry {
    ytgb_render_args args;
    int32_t tile_begin;  /* first work item of this view */
    int32_t tiles_y;     /* tiles along the image's second axis */
    int32_t tiles;       /* work items of this view */
    int32_t pad;
} ytgb_batch_entry;

/* ---- status -------------------------------------------------------------- */
int ytgb_abi_version(void);
const char *ytgb_last_error(void);
/* reads and clears the device error word written by a render */
int ytgb_check_error(const int32_t *d_error, void *stream);

/* ---- host: pixel culling ------------------------------------------------- */
/* Replaces ImageSampler.extent_function + the +-1 padding and clipping of
 * cast_through_kdtree (image_samplers.pyx:159-163; lenses.pyx:22-175).
 * For each brick order[k] writes rects[4k..4k+3] = {x0, x1, y0, y1}: the
 * half-open pixel range [x0,x1) x [y0,y1) the reference would loop over.
 * `bricks` and `order` are host arrays. */
int ytgb_brick_rects(const ytgb_view *view, const ytgb_brick *bricks, int32_t n_bricks,
                     const int32_t *order, int32_t n_order, int32_t *rects);

/* ---- host: transfer function --------------------------------------------- */
/* Replaces FIT_initialize_table (field_interpolation_tables.pxd:44-61) for the
 * tables of VolumeRenderSampler.__cinit__ (image_samplers.pyx:425-447).
 * values[t] points to nbins[t] float64 values; bounds is 2*n_fits.
 * tables_out must hold n_fits * max(nbins) * 4 floats. */
int ytgb_tf_pack(int32_t n_fits, const double *const *values, const int32_t *nbins,
                 const double *bounds, const int32_t *field_ids, const int32_t *weight_field_ids,
                 const int32_t *weight_table_ids, const int32_t *field_table_ids,
                 int32_t grey_opacity, ytgb_tf *tf_out, float *tables_out);

/* ---- device: rendering --------------------------------------------------- */
/* One view over an ordered brick list; replaces the Python brick loop of
 * KDTreeVolumeSource.render (render_source.py:594-596) calling
 * ImageSampler.__call__ -> cast_through_kdtree -> walk_volume -> sample. */
int ytgb_render(const ytgb_render_args *args, void *stream);

/* Traversal trace: for every pixel, an FNV-1a hash over (brick, index[3],
 * enter_t bits, exit_t bits) of every cell walk_volume (grid_traversal.pyx:
 * 26-140) hands to the sampler, and the visit count.  hashes/counts are
 * device (nx*ny) arrays, initialised by the caller (FNV offset basis, 0). */
int ytgb_trace(const ytgb_render_args *args, unsigned long long *hashes, long long *counts, void *stream);

/* ---- device: many views in one persistent launch ------------------------- */
/* Host: validate a batch (host copy of the entries; all of one sampler kind
 * and kernel variant, YTGB_VARIANT_* below) and number its tiles for a tile
 * shape.  Writes
 * tile_begin / tiles_y / tiles of each entry, the total tiles and the
 * shared memory the launch stages its transfer function in: nonzero only
 * when every entry reads the same tables (same pointer and header); 0 when
 * they differ, and then the launch reads the tables from global memory.
 * The same render as calling ytgb_render for every entry; there is no
 * reference counterpart (yt renders one camera at a time). */
int ytgb_batch_plan(ytgb_batch_entry *entries, int32_t n, int32_t tile_shape, int32_t *total_tiles,
                    int32_t *smem_bytes);
/* The kernel variant of a batch (ytgb_batch_plan requires every entry to
 * call for the same one): YTGB_VARIANT_CTF where the volume-rendering tables
 * are a ColorTransferFunction (tf.ctf_fast), plus YTGB_VARIANT_RANGE64
 * where volume-rendering or light-source entries carry data_lo and
 * range_eps > 0 (float64 range decisions near a bound; not for a
 * ColorTransferFunction whose table excludes every value). */
#define YTGB_VARIANT_CTF 1
#define YTGB_VARIANT_RANGE64 2
/* Device: render a planned batch (entries copied to device memory) with one
 * persistent launch of `blocks` blocks (<= 0: one wave of the GPU) whose
 * warps pull 32-pixel work items from *d_queue, which it resets first.
 * smem_bytes as ytgb_batch_plan wrote it (a staged table too large for it
 * raises YTGB_DEVERR_BAD_TF in the error word instead of rendering).
 * variant: the entries' YTGB_VARIANT_* bits.  Graph-capturable. */
int ytgb_batch_render(const ytgb_batch_entry *d_entries, int32_t n, int32_t kind, int32_t variant,
                      int32_t tile_shape, int32_t total_tiles, int32_t smem_bytes, int32_t *d_queue,
                      int32_t blocks, void *stream);

/* The same render with nothing allocated by the caller or the call: the
 * planned host table (h_entries, from ytgb_batch_plan) is copied into a
 * static device region of this library that also holds the work-queue
 * counter, then the persistent launch runs from there.  No counterpart in
 * the reference (yt renders one camera at a time and allocates per call).
 * The host table is checked against the arguments before anything is
 * queued (each entry's arguments, sampler kind and variant, smem_bytes
 * against the entries' tables, the tile numbering ytgb_batch_plan writes for
 * tile_shape, total_tiles); a mismatch returns YTGB_ERR_INVALID.
 * Limits: at most YTGB_NOALLOC_MAX_ENTRIES views per call (more is rejected
 * with YTGB_ERR_INVALID); the region is per device, so calls on one device
 * must not overlap in time (use one stream, or wait for the previous call's
 * work); the first call on a device looks the region up
 * (cudaGetSymbolAddress) -- make it outside any stream capture -- and keeps
 * the address for the life of the process, so do not call it again on a
 * device after cudaDeviceReset.  h_entries in pageable memory may be reused
 * once the call returns; in page-locked memory (cudaHostAlloc,
 * cudaHostRegister) it is read asynchronously and must stay unchanged until
 * the stream has passed the call.  The counter is cleared by every call;
 * nothing needs to be zero beforehand. */
#define YTGB_NOALLOC_MAX_ENTRIES 128
int ytgb_batch_render_noalloc(const ytgb_batch_entry *h_entries, int32_t n, int32_t kind, int32_t variant,
                              int32_t tile_shape, int32_t total_tiles, int32_t smem_bytes, int32_t blocks,
                              void *stream);

/* ---- device: brick preparation ------------------------------------------ */
/* Replaces the per-leaf host work of AMRKDTree.get_brick_data
 * (amr_kdtree.py:325-374): vertex centring of the leaf's grid
 * (ghost_zone_interpolate without ghost zones, interpolators.pyx:177-226,
 * grid_patch.py:270-296), log10 with values <= 0 -> NaN when log_field, and
 * the slice [li:ri+1], written as float32 into field `field` of each brick's
 * arena slot.  All arrays are device arrays: d_cells holds every grid's
 * float64 cell data (C order) at d_grid_offset[g] with dims d_grid_dims[3g..];
 * brick b takes grid d_brick_grid[b] from vertex d_brick_lo[3b..] with the
 * dims and arena slot of d_bricks[b].  Every index is checked on the device;
 * a brick that does not fit is skipped and YTGB_DEVERR_BAD_BRICK is written
 * to *d_error (read it with ytgb_check_error).  d_arena_lo (or NULL) receives
 * each value's float32 rounding error, laid out like d_arena. */
int ytgb_vertex_bricks(const double *d_cells, int64_t n_cells, const int64_t *d_grid_offset,
                       const int32_t *d_grid_dims, int32_t n_grids, const int32_t *d_brick_grid,
                       const int32_t *d_brick_lo, const ytgb_brick *d_bricks, int32_t n_bricks, int32_t field,
                       int32_t log_field, float *d_arena, int64_t arena_len, int32_t *d_error, void *stream,
                       float *d_arena_lo);

/* ---- host: brick marshalling -------------------------------------------- */
/* No reference counterpart: yt's sampler reads each PartitionedGrid's
 * float64 arrays in place (image_samplers.pyx:146-197, partitioned_grid.pyx:
 * 38-70).  The device path gathers every brick's fields into one float32
 * arena per render: dst[dst_offset[k] + i] = (float)src[k][i] for
 * i < count[k], k < n, on up to n_threads host threads (<= 0: all cores).
 * Round to nearest even, as numpy's astype(float32). */
int ytgb_pack_fields(const double *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n,
                     float *dst, int32_t n_threads);
/* The same gather writing each value's float32 part to dst_hi and its
 * float32 rounding error (value - hi, rounded to float32; 0 for non-finite
 * values) to dst_lo: the low parts the light-source sampler's gradient uses. */
int ytgb_pack_fields_split(const double *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n,
                           float *dst_hi, float *dst_lo, int32_t n_threads);
/* The same gather done by the device, for GPUs that read pageable host
 * memory coherently (cudaDevAttrPageableMemoryAccess, e.g. a Grace CPU
 * joined to its GPU by NVLink-C2C): the kernel reads the host float64 arrays
 * src[k] directly and writes d_arena[dst_offset[k] + i] = (float)src[k][i]
 * for i < count[k], and the low parts into d_arena_lo when it is not NULL
 * (as ytgb_pack_fields_split).  src, count and dst_offset are host arrays,
 * read by the device too; they and the fields must stay unchanged until the
 * stream has passed the launch.  Every destination range is checked against
 * arena_len on the host first.  Returns YTGB_ERR_INVALID, launching
 * nothing, on a device without pageable memory access. */
int ytgb_gather_fields(const double *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n,
                       float *d_arena, float *d_arena_lo, int64_t arena_len, void *stream);
/* The masks' counterpart of ytgb_gather_fields: the device copies the host
 * uint8 masks src[k] (count[k] bytes, of brick brick[k]) to d_masks +
 * dst_offset[k] and sets d_desc[brick[k]].mask_offset = dst_offset[k] for a
 * brick with any byte other than 1 (descriptors keep -1, all ones,
 * otherwise).  Host arrays read by the device, as for ytgb_gather_fields. */
int ytgb_gather_masks(const uint8_t *const *src, const int64_t *count, const int64_t *dst_offset,
                      const int32_t *brick, int64_t n, uint8_t *d_masks, int64_t masks_len, ytgb_brick *d_desc,
                      int32_t n_bricks, void *stream);
/* *out = 1 when the current device reads pageable host memory coherently
 * (the condition of ytgb_gather_fields), else 0. */
int ytgb_device_reads_host(int32_t *out);
/* The same gather for uint8 cell masks (dst may be NULL: check only);
 * *all_ones = 1 when every mask byte is 1 (VolumeRenderSampler then needs no
 * mask, image_samplers.pyx:461-462). */
int ytgb_pack_masks(const uint8_t *const *src, const int64_t *count, const int64_t *dst_offset, int64_t n,
                    uint8_t *dst, int32_t n_threads, int32_t *all_ones);
/* *result = 1 when all n float64 values have the bit pattern of `value`
 * (an all-zero image needs no upload; an all-ones zbuffer equals none). */
int ytgb_host_is_uniform(const double *x, int64_t n, double value, int32_t n_threads, int32_t *result);

/* memcpy on up to n_threads host threads (<= 0: all cores): moves a
 * rendered image from a pinned staging buffer into the caller's array. */
int ytgb_host_copy(void *dst, const void *src, int64_t bytes, int32_t n_threads);

/* Prefault the whole pages of a host array for writing without changing
 * its contents (madvise MADV_POPULATE_WRITE).  A freshly allocated zero
 * image that is read before it is written (the zero check above, yt's own
 * read-modify-write) otherwise maps the kernel's shared zero page first and
 * pays a copy-on-write fault per page on the write: on the Grace host that
 * made writing a 32 MiB image ~12 ms instead of ~0.7 ms. */
int ytgb_host_prefault(void *p, int64_t bytes);

/* ---- octree volumes --------------------------------------------------------- */
/* One node of an octree as built by ytgb_octree_build: children (-1 none,
 * index iflat = 4x + 2y + z of the child octant), the cell key of a terminal
 * node, flags (bit 0 terminal, bit 1 has children). */
typedef struct ytgb_onode {
    int32_t child[8];
    int32_t key;
    int32_t flags;
} ytgb_onode;

/* An octree volume on the device: the nodes, and per cell (key) its 8
 * vertex values (float32, (i,j,k) C order) and 9 float64 edge values (left
 * edge, right edge, 1/(right - left)) -- the 14 values per cell of yt's
 * octree volume source (render_source.py:667-680) split by precision. */
typedef struct ytgb_octree_args {
    const ytgb_onode *nodes;
    const float *verts;
    const double *edges;
    int32_t n_nodes;
    int32_t n_cells;
    int32_t depth;
    int32_t pad;
    double dle[3];
    double dre[3];
    /* optional (NULL: not used): per cell 12 floats -- the left edge split
     * into float32 high and low parts (3 + 3), (float)(1/(right - left)) (3),
     * 3 unused -- from which the samplers form each cell's entry point in
     * float32 pairs instead of float64 (16-byte aligned) */
    const float *edges_f;
} ytgb_octree_args;

/* Replaces _OctreeRayTracing(LE, RE, depth).add_nodes(ipos, lvl, key)
 * (_octree_raytracing.pyx:14-31; Octree::insert_node and create_get_node,
 * _octree_raytracing.hpp:139-175, 238-257): nodes are numbered in creation
 * order, the root first.  Returns a handle (NULL on bad input). */
void *ytgb_octree_build(int32_t depth, const double *dle, const double *dre, const int32_t *ipos,
                        const int32_t *lvl, const int32_t *key, int64_t n);
int64_t ytgb_octree_num_nodes(void *tree);
int ytgb_octree_nodes(void *tree, ytgb_onode *out);
void ytgb_octree_destroy(void *tree);

/* Replaces ImageSampler.cast_through_octree (image_samplers.pyx:202-288):
 * every pixel's ray cast through the octree (Octree::cast_ray,
 * _octree_raytracing.hpp:199-230, 276-366) and each terminal cell handed to
 * the sampler of args->kind as a 1x1x1 brick, in traversal order.  The rays
 * are per-pixel (YTGB_LENS_PER_PIXEL or YTGB_LENS_PERSPECTIVE; the
 * reference reads per-pixel ray arrays).  args->data must be o->verts;
 * bricks, order and rects are unused. */
int ytgb_render_octree(const ytgb_render_args *args, const ytgb_octree_args *o, void *stream);
/* Traversal trace of the octree path: per pixel an FNV-1a hash over (cell
 * key, enter t bits, exit t bits) of every cell sampled, and the count. */
int ytgb_trace_octree(const ytgb_render_args *args, const ytgb_octree_args *o, unsigned long long *hashes,
                      long long *counts, void *stream);

/* ---- octree off-axis projection (cell splatting) ------------------------- */
/* The cells of an octree dataset projected along a rotated axis by
 * splatting (image_utilities.pyx:167-289, add_cells_to_image_offaxis, and
 * its per-cell _add_cell_to_image_offaxis :46-165, called from
 * off_axis_projection.py:434-499): every cell stamps the projected depth of
 * a unit cube, precomputed per resolution level ("stamp", :229-246, by
 * direct_integrate_cube :321-407), onto the pixels it covers, weighted by
 * the cell's quantity and weight and dx^3 * Nx * Ny.  Pixel (i, j) is the
 * element i * nx + j of buffer and buffer_weight (the reference's ij2idx,
 * :43-44), which for nx == ny is the C-order (nx, ny) image; the reference
 * writes outside its (nx, ny) buffers when nx > ny, which is rejected. */
typedef struct ytgb_offaxis_args {
    const double *xp;        /* (n, 3) cell centres, relative to the image centre, in image widths */
    const double *dxp;       /* n cell widths, in image widths */
    const double *qty;       /* n */
    const double *weight;    /* n */
    const double *stamp;     /* (max_depth, nsx, nsy): the stamps, 0 where the stamp mask is 0 */
    double *buffer;          /* nx * ny, accumulated into */
    double *buffer_weight;   /* nx * ny, accumulated into */
    double rot[6];           /* rows 0 and 1 of the rotation (the camera's inverse matrix, transposed) */
    int64_t n;
    int32_t nx, ny;
    int32_t nsx, nsy;        /* the stamp's extent: max(npix_min, ceil(2 sqrt(3) max(dxp) nx)), ... */
    int32_t max_depth;       /* ceil(log2(max(nsx, nsy))) */
    int32_t pad;
} ytgb_offaxis_args;

/* The unnormalised stamps: for every level d in 1 .. max_depth-1 the depth
 * zmax - zmin of the parallelepiped spanned by u, v, w from o at the centres
 * of a min(2^d, nsx) x min(2^d, nsy) grid, and its hit mask
 * (direct_integrate_cube, image_utilities.pyx:321-407, with
 * check_in_parallelogram :296-318), written into stamp / mask (max_depth,
 * nsx, nsy) zeroed by the caller; each level is then divided by its sum.
 * Returns YTGB_ERR_INVALID where the reference raises ("This should not
 * happen": a pixel met by one face). */
int ytgb_offaxis_depths(const double *o, const double *u, const double *v, const double *w, int32_t nsx,
                        int32_t nsy, int32_t max_depth, double *stamp, uint8_t *mask);

/* Replaces add_cells_to_image_offaxis's cell loop (image_utilities.pyx:
 * 249-289): accumulates every cell into buffer / buffer_weight on the
 * device.  All pointers are device pointers; d_error (may be NULL) gets
 * YTGB_DEVERR_BAD_CELL when a cell's stamp index is out of range. */
int ytgb_offaxis_cells(const ytgb_offaxis_args *args, int32_t *d_error, void *stream);

/* ---- host: AMR kd-tree --------------------------------------------------- */
/* Replaces AMRKDTree's Tree.build (amr_kdtree.py:109-118) over
 * amr_kdtools.Node.add_grids / insert_grids / split_grids /
 * kdtree_get_choices / divide (amr_kdtools.pyx:201-532, 760-823).
 * Grids are added level by level in the given order. Returns a handle. */
void *ytgb_kdtree_build(int32_t n_grids, const double *gles, const double *gres,
                        const int64_t *gids, const int32_t *levels);
void ytgb_kdtree_destroy(void *tree);
/* number of leaves with a grid (the bricks) */
int32_t ytgb_kdtree_num_leaves(void *tree);
/* leaves in depth-first (left-first) order: kd_traverse() without viewpoint
 * (amr_kdtools.pyx:102-107) */
int ytgb_kdtree_leaves(void *tree, double *le, double *re, int64_t *grid_ids);
/* leaf indices (into the depth-first list) in the viewpoint order of
 * kd_traverse(viewpoint) (amr_kdtools.pyx:108-111, 612-622, 708-755) */
int ytgb_kdtree_viewpoint_order(void *tree, const double *viewpoint, int32_t *order);
/* the same for many viewpoints: order is n_views * num_leaves */
int ytgb_kdtree_viewpoint_orders(void *tree, int32_t n_views, const double *viewpoints, int32_t *order);

#ifdef __cplusplus
}
#endif
#endif /* YTGB_H */
