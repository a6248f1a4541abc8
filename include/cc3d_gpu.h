/*
 * cc3d_gpu.h -- C ABI of the GB300 labelling core (libcc3d_gpu.so).
 *
 * Drop-in boundary for cc3d's labelling hot path.  Each entry point names the
 * reference interface it replaces (paths relative to the cc3d source tree).
 * Plain pointers and sizes only; no exceptions cross this boundary.
 *
 * Conventions
 *   - Return CC3D_OK (0) or a negative CC3D_ERR_*; cc3d_gpu_last_error()
 *     returns the message of the last failure on the calling thread.
 *   - Volumes are raster ordered with x fastest: voxel (x, y, z) lives at
 *     x + sx * (y + sy * z), as the reference's C++ core sees them after the
 *     Cython layer has reversed C-order shapes (cc3d/fastcc3d.pyx:352-359).
 *   - `mem_flags` says where each buffer lives: CC3D_IN_DEVICE and/or
 *     CC3D_OUT_DEVICE.  Host buffers are staged through device memory owned by
 *     the library; device buffers are used in place.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     ordered on that stream and return after the results they report (N,
 *     counts, errors) are known, so host output buffers are filled on return.
 *   - Calls may come from several host threads at once: every thread uses its
 *     own device workspace.
 *   - Volumes whose row-padded voxel count (ceil(sx/32)*32 * sy * sz) reaches
 *     2^32 are rejected with CC3D_ERR_UNSUPPORTED.
 */
#ifndef CC3D_GPU_H
#define CC3D_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element types (signed integers are passed as the unsigned type of the same
   width, float16 as uint16, bool as uint8, exactly as the reference's Cython
   layer views them: cc3d/fastcc3d.pyx:346-350, 494-608) */
#define CC3D_U8 1
#define CC3D_U16 2
#define CC3D_U32 3
#define CC3D_U64 4
#define CC3D_F32 5
#define CC3D_F64 6

#define CC3D_IN_DEVICE 1
#define CC3D_OUT_DEVICE 2

#define CC3D_OK 0
#define CC3D_ERR_INVALID -1      /* bad argument (ValueError in cc3d)              */
#define CC3D_ERR_UNSUPPORTED -2  /* outside what this library implements            */
#define CC3D_ERR_CUDA -3         /* a CUDA runtime call failed                       */
#define CC3D_ERR_NOMEM -4        /* device allocation failed                         */
#define CC3D_ERR_RUNTIME -5      /* the reference's std::runtime_error cases         */
#define CC3D_ERR_DEVICE -6       /* a kernel gave up (iteration budget) and reported */
#define CC3D_ERR_OVERFLOW -7     /* value does not fit a C int64 (OverflowError)     */
#define CC3D_ERR_NAN -8          /* NaN where the reference converts to int64        */

const char* cc3d_gpu_last_error(void);
const char* cc3d_gpu_version(void);

/*
 * Estimated provisional label count and first/last foreground row.
 * Replaces cc3d::estimate_provisional_label_count<T>
 * (cc3d/cc3d.hpp:287-315; bound at cc3d/fastcc3d.pyx:60-65, called from
 * estimate_provisional_labels, cc3d/fastcc3d.pyx:168-242).
 * first_row / last_row are -1 when there is no foreground.
 */
int cc3d_gpu_estimate_provisional_label_count(
    const void* in, int dtype, int64_t sx, int64_t voxels,
    uint64_t* epl, int64_t* first_row, int64_t* last_row,
    int mem_flags, void* stream);

/*
 * Connected components of `in` into `out` (uint16/32/64 by out_dtype).
 * Replaces cc3d::connected_components3d<T,OUT>(in, sx, sy, sz, max_labels,
 * connectivity, delta, out, N, periodic_boundary, binary_image)
 * (cc3d/cc3d_continuous.hpp:394-455; bound at cc3d/fastcc3d.pyx:67-74).
 *   connectivity: 26, 18, 6, or 8, 4 (the latter two need sz == 1, else
 *                 CC3D_ERR_RUNTIME "sz must be 1 for 2D connectivities.").
 *   max_labels:   the Cython layer's estimate; it only matters for binary
 *                 images, where the reference's union-find is sized from it
 *                 and throws "maximum length exception" when too small -- this
 *                 library reports that case as CC3D_ERR_RUNTIME too.
 *   delta:        0, or continuous labelling (cc3d/cc3d_continuous.hpp:90-392)
 *                 with delta converted to the element type (exact for
 *                 integers below 2^53; cc3d_gpu_label_prepare_continuous takes
 *                 an element).  Ignored for binary images.
 * Labels are numbered 1..N in raster order of each component's first voxel;
 * binary 8-connected images are numbered in raster order of each component's
 * first 2x2 block, as the reference's block labeller does.  Background is 0.
 */
int cc3d_gpu_connected_components3d(
    const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
    int64_t max_labels, int64_t connectivity, double delta,
    void* out, int out_dtype, uint64_t* N,
    int periodic_boundary, int binary_image,
    int mem_flags, void* stream);

/*
 * The same labelling in two steps, for callers that choose the output dtype
 * from the provisional-label estimate, as the reference's Cython layer does
 * (cc3d/fastcc3d.pyx:386-434): the estimate is computed in the same pass over
 * the input as the labelling, so the volume is read once.
 *
 * cc3d_gpu_label_prepare runs every stage up to the numbering and returns the
 * estimate (epl, first/last foreground row; for binary images the values the
 * Cython layer substitutes: voxels, 0, sy), the number of components N and a
 * token.  cc3d_gpu_label_finish(token, ...) then writes the labels in the
 * chosen dtype; it must be called on the same thread before any other call of
 * this library on that thread.  max_labels and the error cases are as for
 * cc3d_gpu_connected_components3d.
 */
typedef struct {
  uint64_t token;
  uint64_t epl;
  int64_t first_row;
  int64_t last_row;
  uint64_t N;
  uint64_t provisional;  /* provisional labels the reference's binary labeller opens */
  uint64_t edges;        /* tile-boundary edges merged (a measure of boundary work) */
} cc3d_gpu_prepared;

int cc3d_gpu_label_prepare(
    const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
    int64_t connectivity, int periodic_boundary, int binary_image,
    int mem_flags, void* stream, cc3d_gpu_prepared* info);

/*
 * The continuous-value labelling, first step (finish with
 * cc3d_gpu_label_finish).  Replaces cc3d::connected_components3d<T,OUT> with
 * delta != 0 (cc3d/cc3d_continuous.hpp:394-455 -> 90-392): neighbours join
 * when both are foreground and |a - b| <= delta in the element type (unsigned
 * without underflow; floating point by the rounded difference, so NaN joins
 * nothing).  26/18/6 use the 3D labeller for any sz; 4 the 2D 4-connected one;
 * 8 the 2D 8-connected one including its decision tree, where a pixel takes
 * the label of the pixel above when both lie within delta of the image's
 * minimum and maximum (cc3d/cc3d_continuous.hpp:296-309).  `delta` points to
 * one element of the input type.  The result is numbered like every other
 * path (raster order of each component's first voxel); periodic boundaries
 * are not supported (CC3D_ERR_RUNTIME, as the reference throws).
 */
int cc3d_gpu_label_prepare_continuous(
    const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
    int64_t connectivity, const void* delta, int mem_flags, void* stream,
    cc3d_gpu_prepared* info);

/*
 * Connected components of a voxel connectivity graph, first step (finish with
 * cc3d_gpu_label_finish, uint32 output).  Replaces color_connectivity_graph_N
 * (cc3d/cc3d_graphs.hpp:1077-1105, bound at cc3d/fastcc3d.pyx:941-1019):
 * every voxel is a node, and a voxel joins a backward neighbour (inside the
 * volume) when its own bit for that direction is set, so an asymmetric graph
 * follows the later voxel's bits as the reference does.  `vcg` is uint8 or
 * uint32 (dtype CC3D_U8 / CC3D_U32).  With sz > 1 connectivity is 6 or 26 (3D
 * bit layout); a single plane is 4-connected for 4 and 6 and 8-connected for
 * 8 and 26, reading uint8 graphs in the 2D layout and uint32 graphs in the 3D
 * one, as the reference's two 8-connected labellers do.  Components are numbered 1..N in raster order of
 * their first voxel.
 */
int cc3d_gpu_label_prepare_graph(
    const void* vcg, int dtype, int64_t sx, int64_t sy, int64_t sz,
    int64_t connectivity, int mem_flags, void* stream, cc3d_gpu_prepared* info);

int cc3d_gpu_label_finish(
    uint64_t token, int64_t max_labels, void* out, int out_dtype, uint64_t* N,
    int mem_flags, void* stream);

/*
 * The single-foreground-row case of the Cython layer: the foreground row
 * `row` (0-based over sy*sz rows) is labelled run by run, keeping the previous
 * run's value in a C int64 as the reference does.  Writes only that row of
 * `out` (the caller zero-fills the rest, as np.zeros does in the reference).
 * Replaces epl_special_row (cc3d/fastcc3d.pyx:644-679, called at :469-470).
 * Returns CC3D_ERR_NAN / CC3D_ERR_OVERFLOW where the reference raises
 * ValueError / OverflowError converting a run value to int64; `is_uint64`
 * marks unsigned 64-bit input (values >= 2^63 overflow).
 */
int cc3d_gpu_special_row(
    const void* in, int dtype, int is_uint64, int64_t sx, int64_t sy, int64_t sz,
    int64_t row, void* out, int out_dtype, uint64_t* N, int mem_flags, void* stream);

/*
 * Largest and smallest label value (the N and sign checks of statistics,
 * cc3d/fastcc3d.pyx:731-747).  `is_signed` interprets the element bits as
 * two's complement; results are returned as int64 bit patterns in *vmax/*vmin
 * (for unsigned 64-bit input *vmax is the raw uint64 value).
 */
int cc3d_gpu_label_minmax(
    const void* labels, int dtype, int is_signed, int64_t voxels,
    uint64_t* vmax, int64_t* vmin, int mem_flags, void* stream);

/*
 * Per-label voxel counts, bounding boxes and centroids.
 * Replaces _statistics_helper2d/_statistics_helper3d
 * (cc3d/fastcc3d.pyx:767-844, 846-938).
 *   Dimensions d0, d1, d2 are the numpy axes (x = axis 0, y = axis 1,
 *   z = axis 2; d2 = 1 and ndim = 2 for images); `c_order` says whether the
 *   last axis (1) or the first axis (0) is fastest in memory.
 *   counts:    uint32[N+1]
 *   bboxes:    uint16 or uint32 (bbox_dtype CC3D_U16/CC3D_U32) [N+1][2*ndim],
 *              (min, max) per axis; mins start at the type's maximum.
 *   centroids: float64 [N+1][ndim]; NaN where the count is 0.
 * Output buffers are host or device memory per CC3D_OUT_DEVICE.
 * N must be at least the largest label (the reference computes it as the
 * maximum); voxels whose label exceeds N are skipped and the call returns
 * CC3D_ERR_DEVICE.
 */
int cc3d_gpu_statistics(
    const void* labels, int dtype, int64_t d0, int64_t d1, int64_t d2,
    int ndim, int c_order, uint64_t N,
    uint32_t* counts, void* bboxes, int bbox_dtype, double* centroids,
    int mem_flags, void* stream);

/*
 * Per-stage timing of this thread's calls, measured with CUDA events on the
 * call's own stream (no reference counterpart: the reference has no device
 * stages).  While enabled, every call adds the milliseconds of each stage to
 * the accumulators below; cc3d_gpu_profile_read copies them (and the number
 * of launches of each stage) and resets them.
 * Stage order: 0 h2d, 1 epl, 2 tile_local, 3 merge_edges, 4 wrap_pairs,
 *              5 scan, 6 write, 7 d2h.
 */
#define CC3D_PROFILE_STAGES 8
void cc3d_gpu_profile_enable(int enable);
int cc3d_gpu_profile_read(double* ms, uint64_t* launches, int n);

/*
 * Iteration budget of every bounded union-find loop on the device (the find,
 * union and tile-union loops of the labelling kernels), for all threads of
 * the process; 0 (the default) restores the built-in limits.  A labelling
 * whose loops run out of budget stops them, skips the rest of their work and
 * returns CC3D_ERR_DEVICE ("... union budget ..." / "find budget"); the GPU
 * stays usable and the next call with an adequate budget is exact.  For
 * testing the give-up path: the reference has no counterpart (its
 * DisjointSet throws when its label array is full, cc3d/cc3d.hpp:107-111).
 * Returns the previous budget, or CC3D_ERR_INVALID for a negative one.
 */
int cc3d_gpu_set_union_budget(int budget);

/* Release this thread's cached device workspace. */
void cc3d_gpu_release_workspace(void);

/*
 * Per-label rewrites of a labelled DEVICE volume: the element-wise halves of
 * cc3d.dust (cc3d/__init__.py:71-155) and cc3d.largest_k
 * (cc3d/__init__.py:199-279), whose per-label decisions the caller makes on
 * the count table (cc3d_gpu_statistics).  Element types are given by their
 * width in bytes (1, 2, 4, 8); labels are unsigned.  A label at or beyond
 * table_len is an error (CC3D_ERR_INVALID).  Ordered on `stream`; return when
 * done.
 *   cc3d_gpu_remap_labels: out[i] = table[labels[i]] (largest_k's
 *     renumbering, or a 0/1 mask for k = 1).
 *   cc3d_gpu_zero_labels: image[i] = 0 where zero[labels[i]] != 0 (dust).
 */
int cc3d_gpu_remap_labels(const void* labels, int label_bytes, int64_t voxels, const void* table,
                          int table_bytes, uint64_t table_len, void* out, void* stream);
int cc3d_gpu_zero_labels(void* image, int image_bytes, const void* labels, int label_bytes,
                         int64_t voxels, const uint8_t* zero, uint64_t table_len, void* stream);

/*
 * Region adjacency of a labelled DEVICE volume (x fastest; labels of
 * label_bytes = 1, 2, 4 or 8, values below 2^32): the counting half of
 * cc3d.contacts / cc3d.region_graph (cc3d/fastcc3d.pyx:1180-1256,
 * cc3d/cc3d_graphs.hpp:238-466), with the reference's neighbourhood at the
 * volume's faces.  cc3d_gpu_contacts counts, for every pair of touching
 * nonzero labels (low, high), its contacts in four classes -- x face, y face,
 * z face, edge or corner -- and returns the number of pairs;
 * cc3d_gpu_contacts_copy then copies the pairs (low << 32 | high) and their
 * four counts (uint32 [npairs][4]) to host memory.  The caller turns counts
 * into areas (faces weigh wy*wz, wx*wz, wx*wy; 2D faces wy, wx; edges and
 * corners 0; or 1 each for voxel counts).  Errors: 2D connectivities with
 * sz != 1 (CC3D_ERR_RUNTIME, the reference's message), labels >= 2^32
 * (CC3D_ERR_UNSUPPORTED).
 */
int cc3d_gpu_contacts(const void* labels, int label_bytes, int64_t sx, int64_t sy, int64_t sz,
                      int64_t connectivity, uint64_t* npairs, void* stream);
int cc3d_gpu_contacts_copy(uint64_t* pairs, uint32_t* counts, uint64_t npairs);

/*
 * Run starts of a labelled DEVICE array in memory order: the device half of
 * cc3d.runs (cc3d/fastcc3d.pyx:1258-1277; extract_runs,
 * cc3d/cc3d_graphs.hpp:470-502).  Position 0 and every position whose label
 * differs from the previous element start a run; cc3d_gpu_run_starts returns
 * their number and cc3d_gpu_run_starts_copy copies the positions (ascending)
 * and the label at each to host memory.  Consecutive starts bound a run; the
 * caller drops runs of label 0.
 */
int cc3d_gpu_run_starts(const void* labels, int label_bytes, int64_t voxels, uint64_t* nstarts,
                        void* stream);
int cc3d_gpu_run_starts_copy(uint64_t* positions, uint64_t* labels, uint64_t nstarts);

/*
 * The seam merge of cc3d.connected_components_stack on the device
 * (cc3d/__init__.py:324-501; the reference's DisjointSet at :296-321, its
 * seam loops at :425-463 and the final crackle.renumber at :488-495).  The
 * caller labels every slab on its own (local labels 1..n_k) and gives slab k
 * the global labels offset_k + 1 .. offset_k + n_k, offset_k = n_0 + ... +
 * n_{k-1}; total_labels = the sum of all n_k.  A device work area of
 * cc3d_gpu_stack_work_bytes(total_labels) bytes holds a union-find table
 * over the global labels.
 *   cc3d_gpu_stack_begin: every label is its own group.
 *   cc3d_gpu_stack_seam: joins the groups of every pair of labels that touch
 *     across one seam: the bottom plane (the last plane of slab k-1) against
 *     the top plane (the first plane of slab k).  Planes are sx * sy device
 *     arrays indexed x * sy + y (the reference's image[x, y, z] with z
 *     fixed); the images' dtype code (CC3D_U8..CC3D_F64, or CC3D_F16)
 *     decides equality (value equality for floats, as numpy's ==) unless
 *     binary_image, where both must be nonzero.  Connectivity 6: the voxel
 *     straight across; 26: the 3 x 3 patch across.
 *   cc3d_gpu_stack_number: each group's number is the rank of its smallest
 *     label among all groups' smallest labels (1..N); N is returned.
 *   cc3d_gpu_stack_relabel: out[x, y, z] = number of (offset + labels[x, y,
 *     z]) (0 for label 0) for a slab of sx * sy * sz voxels read and written
 *     with element strides (x, y, z), so a slab lands in place in the whole
 *     volume's output; *has_background (if not null) is set when any voxel
 *     of the slab is 0.
 * Labels outside the table give CC3D_ERR_INVALID; a union-find loop that runs
 * out of its iteration budget gives CC3D_ERR_DEVICE.  number and relabel
 * synchronise `stream`.
 */
#define CC3D_F16 7 /* float16 images: accepted by cc3d_gpu_stack_seam */
uint64_t cc3d_gpu_stack_work_bytes(uint64_t total_labels);
int cc3d_gpu_stack_begin(void* work, uint64_t total_labels, void* stream);
int cc3d_gpu_stack_seam(const void* bottom_img, const void* top_img, int img_dtype,
                        const void* bottom_labels, int bottom_label_bytes, uint64_t bottom_offset,
                        const void* top_labels, int top_label_bytes, uint64_t top_offset, int64_t sx,
                        int64_t sy, int64_t connectivity, int binary_image, void* work,
                        uint64_t total_labels, void* stream);
int cc3d_gpu_stack_number(void* work, uint64_t total_labels, uint64_t* N, void* stream);
int cc3d_gpu_stack_relabel(const void* labels, int label_bytes, const int64_t* label_strides,
                           uint64_t offset, void* out, int out_bytes, const int64_t* out_strides,
                           int64_t sx, int64_t sy, int64_t sz, void* work, uint64_t total_labels,
                           int* has_background, void* stream);

/*
 * Tile-pass configurations and their autotuner.  No counterpart in the
 * reference, which has a single CPU algorithm per connectivity.  Every
 * configuration gives identical labels; they differ only in speed.
 * A configuration code is a variant ORed with a 3D tile shape and a load
 * path:
 *   CC3D_TILE_LIST  one 256-thread block per tile: each row is related to
 *                   its primary neighbour row by one ballot; voxels that
 *                   relation does not decide go to per-warp lists and are
 *                   handled one per lane (multilabel and binary relations;
 *                   the reference's binary 4-connected relation falls back
 *                   to CC3D_TILE_RUNS).
 *   CC3D_TILE_RUNS  one 256-thread block per tile: rows cut into runs by
 *                   ballots, every neighbour row related by ballots, unions
 *                   of overlapping runs in a shared-memory union-find (every
 *                   relation mode).
 *   CC3D_TILE_8x8 / _4x16 / _16x4   3D tiles of 32 x 8 x 8, 32 x 4 x 16 or
 *                   32 x 16 x 4 voxels (x y z).  2D images always use 32 x 64.
 *   CC3D_TILE_PLAIN the tile's box is read by the block's threads with plain
 *                   loads; without it, by one TMA copy where the volume
 *                   allows it (16-byte aligned base and rows).  Batches
 *                   always use plain loads.
 * Binary 8-connected images always use CC3D_TILE_RUNS (2x2-block numbering).
 *
 * cc3d_gpu_set_tile_pass: the calling thread's configuration (CC3D_TILE_AUTO
 *   = the autotuned choice for the volume's class, else LIST | 8x8); returns
 *   the previous setting, or CC3D_ERR_INVALID for an unknown code.
 * cc3d_gpu_tile_pass_choice: the configuration a labelling of this volume
 *   would use now.
 * cc3d_gpu_tile_config: code of configuration `index` in 0..CC3D_TILE_CONFIGS-1:
 *   for each shape (8x8, 4x16, 16x4), for each variant (LIST, RUNS), the
 *   TMA box then the plain-load box: 12 configurations.
 * cc3d_gpu_autotune: times every configuration on `in` (2D: the first four;
 *   best of `repeats` after one warm-up run each), records the fastest for
 *   the volume's class (dtype, effective connectivity, binary or not, voxel
 *   count within a factor of 8) and returns it in *best; ms[index] gets each
 *   configuration's milliseconds (-1 where not timed) when ms is not NULL
 *   (room for CC3D_TILE_CONFIGS doubles).
 * cc3d_gpu_autotune_reset: forget every recorded choice.
 */
#define CC3D_TILE_AUTO 0
#define CC3D_TILE_RUNS 1
#define CC3D_TILE_LIST 2
#define CC3D_TILE_8x8 0x00
#define CC3D_TILE_4x16 0x10
#define CC3D_TILE_16x4 0x20
#define CC3D_TILE_PLAIN 0x100
#define CC3D_TILE_CONFIGS 12
#define CC3D_TILE_MODEL 3   /* policy: the cost model's choice per volume (below) */
int cc3d_gpu_set_tile_pass(int code);
int cc3d_gpu_tile_pass_choice(int dtype, int64_t sx, int64_t sy, int64_t sz,
                              int64_t connectivity, int binary_image);
int cc3d_gpu_tile_config(int index);
int cc3d_gpu_autotune(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                      int64_t connectivity, int binary_image, int mem_flags, void* stream,
                      int repeats, int* best, double* ms);
void cc3d_gpu_autotune_reset(void);

/*
 * Learned cost model.  No counterpart in the reference.  A small FP32 MLP
 * (CC3D_COST_FEATURES -> 64 -> 64 -> CC3D_TILE_CONFIGS, ReLU) predicts the
 * natural log of the milliseconds every tile-pass configuration takes on a
 * volume, from features sampled on the device; it is trained (mini-batch
 * Adam, squared error over the measured outputs) on timings the autotuner
 * produces.  Labels never depend on it.
 *   cc3d_gpu_volume_features: the 16 features of a DEVICE volume: log2 of sx,
 *     sy, sz and of the voxel count; element bytes / 8; connectivity / 26;
 *     binary flag; and from 65,536 sampled voxels: foreground fraction,
 *     log2(1 + distinct values among 4,096 samples) / 12, the fraction of
 *     foreground samples equal to their +x, +y and +z neighbours, padding
 *     waste of 32 in x and of 8 in y and z, and the fraction of foreground
 *     samples that start a run in x.
 *   cc3d_gpu_cost_model_train: X[n][16] features, Y[n][CONFIGS] log-ms (NaN
 *     where not measured); replaces the process's model.
 *   cc3d_gpu_cost_model_predict: Y[n][CONFIGS] predicted log-ms.
 *   cc3d_gpu_cost_model_get / _set: the CC3D_COST_PARAMS floats of the model
 *     (weights, then feature and output normalisation).
 *   cc3d_gpu_cost_model_choose: the predicted fastest configuration for a
 *     device volume; when the predicted runner-up is within `min_margin`
 *     (relative, e.g. 0.05) the model is not confident and the exhaustive
 *     autotuner decides instead (*confident = 0).
 * With cc3d_gpu_set_tile_pass(CC3D_TILE_MODEL), labellings of device volumes
 * use cc3d_gpu_cost_model_choose (margin 0.05) once a model is loaded;
 * otherwise they behave as CC3D_TILE_AUTO.
 */
#define CC3D_COST_FEATURES 16
#define CC3D_COST_PARAMS 6084
int cc3d_gpu_volume_features(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                             int64_t connectivity, int binary_image, int mem_flags, void* stream,
                             float* features);
int cc3d_gpu_cost_model_train(const float* X, const float* Y, int n, int epochs, int batch, float lr,
                              uint64_t seed, float* final_loss);
int cc3d_gpu_cost_model_predict(const float* X, int n, float* Y);
int cc3d_gpu_cost_model_get(float* params, int n);
int cc3d_gpu_cost_model_set(const float* params, int n);
int cc3d_gpu_cost_model_choose(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                               int64_t connectivity, int binary_image, int mem_flags, void* stream,
                               float min_margin, int* choice, int* confident);

/*
 * Batches: many volumes labelled together.  No counterpart in the reference, whose callers
 * loop over cc3d.connected_components (the result of every volume is
 * identical to that call's: labels, N, and the output type the Cython layer
 * would choose, cc3d/fastcc3d.pyx:388-434).
 *   - multilabel only (binary_image = 0, delta = 0), uint8/16/32 volumes of
 *     one dtype, one connectivity; 2D connectivities need sz == 1;
 *   - `in` and `out` are DEVICE buffers; `out` must hold voxels * 4 bytes and
 *     receives uint16 or uint32 labels as results[i].out_dtype says;
 *   - results[i] gets N, the estimate and first/last foreground row of
 *     volume i; empty volumes get N = 0;
 *   - the call returns when the labels are written.  With stream = NULL the
 *     library waits for the legacy default stream, then runs on a stream of
 *     its own (the legacy stream cannot be captured).
 */
typedef struct {
  const void* in;
  void* out;
  int64_t sx, sy, sz;
} cc3d_gpu_volume;

typedef struct {
  uint64_t N;
  uint64_t epl;
  uint64_t provisional;
  int64_t first_row;
  int64_t last_row;
  int32_t out_dtype;   /* CC3D_U16 or CC3D_U32 */
  int32_t status;      /* 0 */
} cc3d_gpu_volume_result;

int cc3d_gpu_label_batch(const cc3d_gpu_volume* volumes, int n, int dtype, int64_t connectivity,
                         cc3d_gpu_volume_result* results, void* stream);
/* How this thread's cc3d_gpu_label_batch runs (returns the previous mode):
 *   CC3D_BATCH_PERSISTENT (the default): ONE cooperative kernel launch walks
 *     every stage over the whole batch (tile pass, its blocks taking tiles
 *     from a device work queue; edge merges, numbering scan, per-volume
 *     results, labels) with bounded grid barriers between
 *     stages; its arguments come from a header uploaded to device memory, so
 *     the launch is captured into a CUDA graph once (per kernel, grid and
 *     workspace) and replayed for batches of any layout.  3D volumes use the
 *     list pass on 32 x 8 x 8 tiles, 2D images 32 x 64.
 *   CC3D_BATCH_STAGED: one launch per stage (the tile-pass configuration from
 *     the autotuner), the stage sequence captured into a CUDA graph per batch
 *     layout (dtype, connectivity, configuration, list of shapes) and replayed
 *     while the layout repeats.
 * cc3d_gpu_autotune_batch times the staged configurations. */
#define CC3D_BATCH_PERSISTENT 0
#define CC3D_BATCH_STAGED 1
int cc3d_gpu_set_batch_mode(int mode);
/* Release this thread's batch workspace and graphs. */
void cc3d_gpu_release_batch(void);
/* Time every tile-pass configuration on this batch (2D: the first two; best
   of `repeats` after the run that captures each graph), record the fastest
   for the batch's class (dtype, connectivity, mean volume size within 8x) and
   return it in *best; ms[index] gets each configuration's milliseconds (-1
   where not timed) when ms is not NULL.  The labels of the last run are left
   in the volumes' outputs and `results`. */
int cc3d_gpu_autotune_batch(const cc3d_gpu_volume* volumes, int n, int dtype, int64_t connectivity,
                            cc3d_gpu_volume_result* results, void* stream, int repeats, int* best,
                            double* ms);

/*
 * Labelling that allocates nothing.  No counterpart in the reference: the
 * reference labels on the CPU into a buffer its caller allocated and needs no
 * device scratch.
 *
 * Same arguments, results and errors as cc3d_gpu_connected_components3d with
 * delta = 0, for DEVICE input and output buffers only.  Instead of the
 * per-thread workspace the other entry points grow with cudaMalloc, all
 * scratch comes from one fixed array of CC3D_NOALLOC_SCRATCH_BYTES that is part
 * of the library's device image, held by every GPU that loads the library
 * until the process exits.  For callers that cannot allocate device memory
 * while they label: memory owned by another allocator's pool, a fixed memory
 * budget, or loops where cudaMalloc/cudaFree latency and cudaFree's
 * device-wide wait are not acceptable.
 *   - Limit: the scratch of a volume is about 37 KB per 32x8x8 tile (3D) or
 *     31 KB per 32x64 tile (2D), so 128x128x128 (1024 tiles) fits; a larger
 *     volume returns CC3D_ERR_INVALID with the bytes it would need.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - Every call uses the same array, which keeps the last call's contents;
 *     calls whose GPU work overlaps (other threads, unordered streams) race
 *     and corrupt each other's results.
 *   - Allocates no device or pinned memory; N and the device error word come
 *     back through host stack memory, and the call synchronizes `stream`
 *     before it returns, with the labels written.
 */
#define CC3D_NOALLOC_SCRATCH_BYTES 41943040u /* 40 MiB */
int cc3d_gpu_connected_components3d_noalloc(
    const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
    int64_t max_labels, int64_t connectivity,
    void* out, int out_dtype, uint64_t* N,
    int periodic_boundary, int binary_image, void* stream);

/*
 * The voxel connectivity graph of a labelled volume (device pointers): per
 * voxel a bitfield of the directions whose neighbour lies in the volume with
 * the same label or lies outside it.  Replaces
 * extract_voxel_connectivity_graph<T,OUT> (cc3d/cc3d_graphs.hpp:31-240,
 * bound at cc3d/fastcc3d.pyx:1021-1178).  `labels` holds sx*sy*sz unsigned
 * integers of label_bytes (1, 2, 4, 8); sx, sy, sz are the memory extents,
 * fastest first.  With reversed_axes == 0 memory runs x fastest (the
 * reference's Fortran order: x is the array's first axis); with 3 (a 3D
 * array) or 2 (a 2D array) the array is C-ordered, its axes stored in
 * reverse, so the extents are those of (z, y, x) or (y, x, 1) -- and the
 * field is still the reference's.
 * `graph` receives, in the same memory order, uint8 fields for connectivity
 * 4, 8 and 6 and uint32 fields for 18 and 26 (bit layout of the reference:
 * 2D +x -x +y -y xy -xy x-y -x-y; 3D faces, edges, corners).  4 and 8 need
 * sz == 1.  Synchronises `stream`.
 */
int cc3d_gpu_voxel_connectivity_graph(
    const void* labels, int label_bytes, int64_t sx, int64_t sy, int64_t sz,
    int connectivity, int reversed_axes, void* graph, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CC3D_GPU_H */
