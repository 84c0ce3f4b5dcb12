/*
 * vhsdf.h - C ABI of the GB300 voxel-hashing TSDF engine.
 *
 * One handle owns one TSDF volume on one GPU: a lock-free open-addressed
 * spatial hash of 8^3 voxel blocks, the block pool behind it, the per-frame
 * block list, image staging buffers and the triangle buffer of the last
 * marching-cubes extraction.  All entry points return a vh_status; nothing
 * throws across the ABI and nothing exits the process.
 *
 * Each entry point names the reference interface it replaces
 * (E-BAO/Voxel-Hashing-SDF, paths relative to that project).
 *
 * Threading: calls on one handle must be serialised by the caller; different
 * handles are independent.  Work is enqueued on the handle's CUDA stream.
 * Every call works on the handle's GPU (vh_params.device) whatever device
 * the calling thread has current, and leaves that setting unchanged.
 * With VH_FLAG_SYNC set (the default) every call that enqueues work waits
 * for it and reports device-side errors before returning, like the
 * reference's processFrame, which ends in blocking copies.
 */
#ifndef VHSDF_H
#define VHSDF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VHSDF_ABI_VERSION 1

typedef enum vh_status {
  VH_OK = 0,
  VH_ERR_INVALID_ARG = 1,     /* bad pointer, size or parameter            */
  VH_ERR_CUDA = 2,            /* a CUDA runtime call failed                */
  VH_ERR_TABLE_FULL = 3,      /* a hash probe sequence hit max_probe        */
  VH_ERR_POOL_FULL = 4,       /* the voxel-block pool is exhausted          */
  VH_ERR_RETRY_EXHAUSTED = 5, /* a bounded device wait gave up              */
  VH_ERR_NOT_FINITE = 6,      /* non-finite pose or intrinsics              */
  VH_ERR_UNSUPPORTED = 7,     /* feature not available (e.g. GL render)     */
  VH_ERR_OUT_OF_RANGE = 8,    /* block coordinate outside the key range     */
  VH_ERR_CAPACITY = 9,        /* an output buffer is too small              */
  VH_ERR_IO = 10,             /* file could not be read or written          */
  VH_ERR_NO_DEVICE = 11,      /* no CUDA device                             */
  VH_ERR_CHECK = 12           /* a bounds check of the checked build failed */
} vh_status;

typedef enum vh_depth_fmt {
  VH_DEPTH_U16_MM = 0, /* uint16, scaled by depth_scale (0.001 = millimetres) */
  VH_DEPTH_F32_M = 1   /* float32 metres, the processFrame format             */
} vh_depth_fmt;

typedef enum vh_mem {
  VH_MEM_HOST = 0,  /* pointer is host memory (pinned or pageable)            */
  VH_MEM_DEVICE = 1 /* pointer is device memory of the handle's GPU           */
} vh_mem;

typedef enum vh_scope {
  VH_SCOPE_FRAME = 0, /* blocks touched by the last integrated frame          */
  VH_SCOPE_ALL = 1    /* every allocated block (full-volume extraction)       */
} vh_scope;

/* vh_params.flags */
#define VH_FLAG_SYNC 0x1u      /* wait for device work inside every call     */
#define VH_FLAG_NO_GRAPH 0x2u  /* launch kernels directly, no CUDA graphs    */
#define VH_FLAG_PROFILE 0x4u   /* record per-stage CUDA events               */
#define VH_FLAG_DEPTH_FILTER 0x8u /* bilateral pre-filter of every depth    */
                                  /* frame (not the reference's rule; see    */
                                  /* vh_filter_depth)                        */
#define VH_FLAG_BATCH_FUSED 0x10u /* batches only (scene 0's flags): a step */
                                  /* is one persistent launch over every     */
                                  /* stage of every scene (vh_batch_create)  */

/*
 * Volume and camera parameters.  Replaces the arguments of
 * ark::GpuTsdfGenerator::GpuTsdfGenerator (include/tsdf.cuh:606-607,
 * src/tsdf.cu:1248-1372) and the fields of ark::MarchingCubeParam
 * (include/tsdf.cuh:220-233), plus the hash sizes that the reference
 * hard-codes in processFrame (src/tsdf.cu:1488,1492).
 */
typedef struct vh_params {
  int32_t width, height;     /* image size in pixels                        */
  float fx, fy, cx, cy;      /* pinhole intrinsics, pixel centres at ints   */
  float min_depth;           /* near end of a truncation band (m)           */
  float max_depth;           /* depth beyond this is ignored (m)            */
  float depth_scale;         /* metres per VH_DEPTH_U16_MM unit             */
  float voxel_size;          /* voxel edge (m)                              */
  float trunc;               /* truncation margin T (m)                     */
  float mc_min_weight;       /* MC skips cubes with a corner weight below   */
  int32_t table_log2;        /* hash slots = 2^table_log2                   */
  int32_t max_probe;         /* bound on one linear-probe sequence          */
  int64_t pool_blocks;       /* capacity of the voxel-block pool            */
  int64_t max_frame_blocks;  /* capacity of the per-frame block list        */
  int64_t max_triangles;     /* initial capacity of the triangle buffer     */
  uint32_t flags;            /* VH_FLAG_*                                   */
  int32_t device;            /* CUDA device ordinal                         */
} vh_params;

/* Block-edge length in voxels of every volume (fixed for this ABI). */
#define VH_BLOCK_EDGE 8
#define VH_BLOCK_VOXELS 512

typedef struct vh_stats {
  int64_t frames;            /* frames integrated since create/reset        */
  int64_t blocks_allocated;  /* live blocks in the pool                     */
  int64_t frame_blocks;      /* blocks in the last frame's block list       */
  int64_t new_blocks;        /* blocks inserted by the last frame           */
  int64_t voxels_updated;    /* voxel updates of the last frame             */
  int64_t triangles;         /* triangles of the last extraction            */
  int64_t pool_capacity;
  int64_t table_slots;
  int64_t tombstones;        /* erased hash slots not yet reclaimed         */
  uint32_t device_error;     /* sticky device error bits (0 = none)         */
  uint32_t frame_kernels;    /* kernels launched by the last frame          */
  /* per-stage device time of the last frame in ms (VH_FLAG_PROFILE only)   */
  float ms_allocate, ms_integrate, ms_extract, ms_frame;
} vh_stats;

/* A device-resident triangle soup: triangle t has vertices 3t..3t+2, each a
 * float4 {x, y, z, rgb} in global voxel units (multiply by voxel_size for
 * metres, as the reference's tsdf2mesh does, src/tsdf.cu:1815-1817); the
 * fourth float holds the colour bytes r | g<<8 | b<<16.  Valid until the
 * next call on the handle. */
typedef struct vh_mesh_view {
  const float *vertices;     /* device pointer, 12 floats per triangle      */
  int64_t num_triangles;
  float voxel_size;
} vh_mesh_view;

/* Launch configuration of the per-frame kernels.  Every configuration
 * computes identical results; only the speed differs. */
typedef struct vh_tuning {
  int32_t integrate_variant;     /* voxels per thread x threads per CTA,     */
                                 /* register budget (CTAs per SM):           */
                                 /* 0: 4 x 128, 12   1: 4 x 128, next block  */
                                 /*    prefetched, 8   2: 8 x 64, 16         */
                                 /* 3: 2 x 256, 6   4: 4 x 128, 10           */
                                 /* 5: 8 x 64, 12                            */
  int32_t integrate_ctas_per_sm; /* resident CTAs per SM (0 = occupancy max) */
  int32_t mc_ctas_per_sm;        /* resident CTAs per SM (0 = occupancy max) */
  int32_t mc_variant;            /* 0: register budget for 10 CTAs per SM,   */
                                 /* 1: for 12 CTAs per SM                    */
} vh_tuning;

typedef struct vh_handle vh_handle;

/* ---- parameters --------------------------------------------------------- */

/* Defaults of the reference's scene YAML where it has one
 * (scene0220_02/scene0220_02.yaml:12-15,21-22,37-62; min_depth 0.1 from
 * src/tsdf.cu:1318), 8^3 blocks, 2^20 hash slots. Host only. */
vh_status vh_params_default(vh_params *p);
/* Checks a parameter set without touching the GPU. Host only. */
vh_status vh_params_validate(const vh_params *p);
const char *vh_status_string(vh_status s);

/* ---- life cycle (ark::GpuTsdfGenerator) ---------------------------------- */

/* Replaces GpuTsdfGenerator::GpuTsdfGenerator (src/tsdf.cu:1248-1372) and
 * vhashing::HashTable::HashTable (include/vhashing.h:643-684). */
vh_status vh_create(const vh_params *p, vh_handle **out);
/* Replaces GpuTsdfGenerator::Shutdown (src/tsdf.cu:1620-1638). */
vh_status vh_destroy(vh_handle *h);
/* Clears the volume (all blocks, the hash and counters). */
vh_status vh_reset(vh_handle *h);
/* Uses cudaStream_t `stream` (NULL = the handle's own stream). */
vh_status vh_set_stream(vh_handle *h, void *stream);
/* Waits for the handle's stream and reports sticky device errors. */
vh_status vh_sync(vh_handle *h);
const char *vh_last_error(const vh_handle *h);

/* Log sink (the reference prints errors with std::cout and glog,
 * src/safecall.cpp:18-53).  fn(level, message, user) receives every error
 * the library records on a handle (the text vh_last_error returns; sticky
 * device errors when vh_sync or vh_get_stats reports them) or on a batch
 * call, and the failures of vh_create before a handle exists.  level is VH_LOG_ERROR.  Process-wide; fn = NULL turns it off.
 * fn runs on the thread that hit the error, possibly on several threads at
 * once, and must not call back into the library.  Host only. */
#define VH_LOG_ERROR 2
typedef void (*vh_log_fn)(int32_t level, const char *message, void *user);
void vh_set_log_callback(vh_log_fn fn, void *user);

/* ---- per-frame path (GpuTsdfGenerator::processFrame) ---------------------- */

/* Allocation + integration of one frame: replaces the HashAssign and
 * IntegrateHashKernel steps of GpuTsdfGenerator::processFrame
 * (src/tsdf.cu:1484-1533, kernels src/tsdf.cu:2088-2238 and 599-751).
 * depth: H*W row-major in `depth_fmt`; rgb: H*W*3 interleaved RGB bytes;
 * c2w: 16 floats, row-major camera-to-world, host memory
 * (PointCloudGenerator.cpp:118-127 builds it this way).
 * VH_MEM_DEVICE images are read in place by the frame's kernels: without
 * VH_FLAG_SYNC they must stay unchanged until the handle's stream has run
 * the frame.  VH_MEM_HOST images are copied on the handle's copy stream
 * into one of two staging slots, overlapping the previous frame's kernels;
 * pinned host memory keeps the call asynchronous (pageable memory is copied
 * before the call returns). */
vh_status vh_integrate(vh_handle *h, const void *depth, int32_t depth_fmt,
                       const uint8_t *rgb, const float *c2w, int32_t mem);
/* Marching cubes over `scope`: replaces marchingCubeHashKernel
 * (src/tsdf.cu:884-1110) for VH_SCOPE_FRAME and the volume walk of
 * tsdf2mesh (src/tsdf.cu:1760-1832) for VH_SCOPE_ALL. `out` may be NULL. */
vh_status vh_extract(vh_handle *h, int32_t scope, vh_mesh_view *out);
/* vh_integrate followed by vh_extract(VH_SCOPE_FRAME): the whole of
 * GpuTsdfGenerator::processFrame (src/tsdf.cu:1484-1598). */
vh_status vh_process_frame(vh_handle *h, const void *depth, int32_t depth_fmt,
                           const uint8_t *rgb, const float *c2w, int32_t mem,
                           vh_mesh_view *out);
/* vh_process_frame with the frame's triangles delivered to host memory, as
 * processFrame copies its triangle buffer back every frame
 * (src/tsdf.cu:1554-1564): tris receives min(n, capacity) triangles in the
 * vh_mesh_view layout (12 floats each) and *num_triangles the frame's count
 * n.  With VH_FLAG_SYNC both are written before the call returns.
 * Otherwise the call returns once the frame is enqueued: the next
 * vh_process_frame_mesh call (after enqueuing its own frame, so the copy
 * overlaps that frame's kernels) or vh_sync writes *num_triangles and issues
 * the copy-out, and a frame's triangles are complete in `tris` once the
 * second vh_process_frame_mesh call after it, or vh_sync, has returned.
 * Until then `tris` and `num_triangles` must stay valid (three host buffers
 * used in turn are enough for a stream of frames).  Pinned host memory keeps
 * the copy asynchronous.  A mesh larger than `capacity` is truncated and
 * reported as VH_ERR_CAPACITY (by vh_sync when asynchronous).  Two device
 * triangle buffers of max_triangles each are added on first use. */
vh_status vh_process_frame_mesh(vh_handle *h, const void *depth, int32_t depth_fmt,
                                const uint8_t *rgb, const float *c2w, int32_t mem, float *tris,
                                int64_t capacity, int64_t *num_triangles);
/* vh_process_frame_mesh with the frame's mesh delivered indexed - the
 * per-frame triangle copy of processFrame (src/tsdf.cu:1554-1564) in
 * another layout: vertices
 * (4 floats each: x, y, z in global voxel units and the colour bytes
 * r | g<<8 | b<<16 in the fourth float's bits, as vh_mesh_view) and faces
 * (3 int32 vertex numbers each).  The faces are exactly the triangles
 * vh_process_frame_mesh delivers (same vertices bit for bit, in another
 * order); marching cubes interpolates each cut lattice edge of a block once
 * and writes its vertex once per block, so a frame's mesh takes about half
 * the bytes of the triangle soup - the copy to host memory is what bounds
 * a stream of frames.  Counts, capacities, the asynchronous protocol
 * (complete after the second call after the frame, or vh_sync) and
 * VH_ERR_CAPACITY follow vh_process_frame_mesh; both buffers stay valid
 * until then.  Two device buffers of max_triangles vertices and faces each
 * are added on first use. */
vh_status vh_process_frame_indexed(vh_handle *h, const void *depth, int32_t depth_fmt,
                                   const uint8_t *rgb, const float *c2w, int32_t mem,
                                   float *vertices, int64_t vertex_capacity, int32_t *faces,
                                   int64_t face_capacity, int64_t *num_vertices,
                                   int64_t *num_faces);
/* Copies the last extraction to host: xyz (9 floats per triangle, voxel
 * units) and rgb (9 bytes per triangle).  Output copies and size queries
 * (all outputs NULL) follow one rule for every copy-out call here: the full
 * count is returned in the count argument, at most `capacity` items are
 * written, and VH_ERR_CAPACITY is returned only when outputs were given and
 * the capacity was too small. */
vh_status vh_copy_mesh(vh_handle *h, float *xyz, uint8_t *rgb,
                       int64_t capacity, int64_t *num_triangles);
/* Full-volume extraction written as PLY with vertices merged by exact
 * position, as GpuTsdfGenerator::SavePLY / tsdf2mesh
 * (src/tsdf.cu:1696-1708,1760-1888). binary = 0 writes the reference's
 * ASCII layout.  The merge runs on the GPU (see vh_mesh_indexed). */
vh_status vh_save_ply(vh_handle *h, const char *path, int32_t binary);
/* Full-volume extraction as an indexed mesh, the data of tsdf2mesh /
 * getVertices / getFaces (src/tsdf.cu:1760-1888, include/tsdf.cuh:631-634):
 * vertices merged by exact position on the GPU and numbered by first
 * occurrence over the triangles sorted by their coordinates (so the result
 * does not depend on GPU scheduling); vertices in metres (3 floats), colours
 * 3 bytes, faces 3 vertex numbers.  NULL outputs: sizes only. */
vh_status vh_mesh_indexed(vh_handle *h, float *vertices, uint8_t *colors, int64_t vertex_capacity,
                          int32_t *faces, int64_t face_capacity, int64_t *num_vertices,
                          int64_t *num_faces);
/* GpuTsdfGenerator::render (src/tsdf.cu:1710-1758) draws with OpenGL; there
 * is no graphics stack here, so this returns VH_ERR_UNSUPPORTED. */
vh_status vh_render(vh_handle *h);

/* ---- hash surface (vhashing::HashTable) ---------------------------------- */

/* Inserts n block keys (int32 x,y,z triples): replaces
 * HashTable::AllocKeys (include/vhashing.h:530-603). Existing keys are kept.
 * Every key is also added to the current block list. */
vh_status vh_alloc_keys(vh_handle *h, const int32_t *xyz, int64_t n,
                        int32_t mem);
/* out_block[i] = pool index of key i or -1: replaces HashTable::find
 * (include/vhashing.h:128-131). */
vh_status vh_find_keys(vh_handle *h, const int32_t *xyz, int64_t n,
                       int32_t *out_block, int32_t mem);
/* Maximum keys per vh_find_keys_noalloc call. */
#define VH_FIND_NOALLOC_MAX_KEYS 65536

/* vh_find_keys for host buffers that allocates no device memory; it has no
 * counterpart in the reference.  For callers that must not call cudaMalloc
 * or cudaFree (a latency-bound loop cannot take cudaFree's device-wide
 * synchronisation; a plugin whose host owns all device memory may not
 * allocate).  xyz and out_block are host memory; out_block[i] is the pool
 * index of key i or -1, as vh_find_keys.  At most VH_FIND_NOALLOC_MAX_KEYS
 * keys per call, else VH_ERR_CAPACITY.  Its scratch is a fixed 1 MiB array
 * that every GPU loading this library holds until the process exits; the
 * first call on a device looks up that array's address, so make the first
 * call before any stream capture.  The address is kept for the life of the
 * process: a cudaDeviceReset of that device invalidates it (and every
 * handle on the device), so do not reset a device this library is using.
 * All calls share the array: calls that
 * overlap on the GPU (other threads, other handles on the same GPU) race and
 * must be serialised by the caller.  The call waits for its result. */
vh_status vh_find_keys_noalloc(vh_handle *h, const int32_t *xyz, int64_t n,
                               int32_t *out_block);
/* Erases n keys and recycles their blocks (zeroed): replaces
 * HashTable::erase (include/vhashing.h:244-256). */
vh_status vh_erase_keys(vh_handle *h, const int32_t *xyz, int64_t n,
                        int64_t *num_erased, int32_t mem);
/* Empties the block list: replaces HashTable::clearheap
 * (include/vhashing.h:80-91). */
vh_status vh_clear_block_list(vh_handle *h);
/* Copies the block list (the reference's key_heap / heap_counter,
 * include/vhashing.h:43,55,417-425) to host int32 triples. */
vh_status vh_block_list(vh_handle *h, int32_t *xyz, int64_t capacity,
                        int64_t *n);
/* The reference's BlockHasher (include/tsdf.cuh:144-156) value of a key. */
uint64_t vh_block_hash_ref(int32_t x, int32_t y, int32_t z);

/* Device addresses of a volume's hash and block pool, for kernels that the
 * caller compiles against include/vhashing_device.cuh: the device members of
 * vhashing::HashTable - operator[] and find (include/vhashing.h:122-135,
 * probe :149-194), Filter (:790-805) and Apply (:818-825) - run as the
 * caller's own device code on these arrays.  The arrays live as long as the
 * handle; their contents are those left by the work enqueued on `stream`
 * before the caller's kernel (order the kernel after it on that stream, or
 * after a synchronising call).  Inserting or erasing keys stays with the
 * library's calls; a caller's kernel may rewrite voxel values of live blocks
 * but must leave slots, keys and ids alone. */
#define VH_DEVICE_TABLE_LAYOUT 1
typedef struct vh_device_table {
  uint32_t layout;            /* VH_DEVICE_TABLE_LAYOUT                       */
  uint32_t slot_mask;         /* slots - 1 (2^table_log2 slots)               */
  int32_t max_probe;          /* bound of one linear probe sequence           */
  int32_t key_bias;           /* packed key: (x + bias) | (y + bias) << 21 |  */
                              /* (z + bias) << 42, coordinates in [-bias, bias) */
  void *slots;                /* 16 B each: uint64 key (all ones empty, all   */
                              /* ones - 1 erased), uint32 pool id, uint32 stamp */
  float *pool;                /* pool_capacity blocks of 3 * 512 words:       */
                              /* sdf[512] | weight[512] | rgba8[512], voxel   */
                              /* index x + 8y + 64z                           */
  const uint64_t *block_keys; /* packed key of every pool block (all ones:    */
                              /* free)                                        */
  const uint32_t *pool_top;   /* device word: ids [0, *pool_top) handed out   */
  int64_t pool_capacity;
  float voxel_size;
  int32_t device;
  void *stream;               /* cudaStream_t of the handle's work when the   */
                              /* table was taken (vh_set_stream changes it)  */
} vh_device_table;
/* Fills *out for handle h.  Host only: enqueues nothing. */
vh_status vh_get_device_table(vh_handle *h, vh_device_table *out);
/* The marching-cubes tables the engine uses, i.e. the reference's
 * MarchingCubeParam idxMap / edgeTable / triTable (include/tsdf.cuh:234-534):
 * corner[8 * 3] voxel offsets of the cube corners, edge_mask[256] cut edges
 * per case, tri[256 * 16] edge triplets per case (-1 padded).  Any output
 * may be NULL. */
vh_status vh_mc_tables(int32_t *corner, int32_t *edge_mask, int32_t *tri);

/* ---- volume I/O ------------------------------------------------------------ */

/* Copies every live block to host (any output may be NULL): keys as int32
 * triples, then per block 512 voxels in x-fastest order (index x + 8y + 64z)
 * of sdf, weight and rgb (3 bytes). Replaces the stream-out copy of
 * getMapValueKernel / streamOutGPU2CPU (src/tsdf.cu:459-596). */
vh_status vh_export_blocks(vh_handle *h, int32_t *xyz, float *sdf,
                           float *weight, uint8_t *rgb, int64_t capacity,
                           int64_t *n);
/* Inserts the given blocks and overwrites their voxels. Replaces the
 * stream-in copy of streamInCPU2GPU (src/tsdf.cu:277-457).  Weights are
 * observation counts, as integration makes them: whole numbers in
 * [0, 2^24], else VH_ERR_INVALID_ARG and nothing is changed. */
vh_status vh_import_blocks(vh_handle *h, const int32_t *xyz, const float *sdf,
                           const float *weight, const uint8_t *rgb, int64_t n);
/* Binary snapshot of the volume (header, keys, voxel payload). */
vh_status vh_save(vh_handle *h, const char *path);
vh_status vh_load(vh_handle *h, const char *path);

vh_status vh_get_stats(vh_handle *h, vh_stats *out);

/* ---- launch tuning (no reference counterpart: the reference launches fixed
 * shapes, src/tsdf.cu:1526-1545,2262-2264) ------------------------------- */

vh_status vh_get_tuning(vh_handle *h, vh_tuning *out);
vh_status vh_set_tuning(vh_handle *h, const vh_tuning *t);
/* Build flags of the loaded library: VH_BUILD_CHECKED when its per-frame
 * kernels were compiled with VH_CHECKED (lib/libvhsdf_checked.so): index
 * checks at every pool, slot, frame-list, pixel and scene access of the
 * allocation, resolve, integration and marching-cubes kernels, which record
 * VH_ERR_CHECK in the device error word and skip the access instead of
 * faulting.  Host only. */
#define VH_BUILD_CHECKED 1u
uint32_t vh_build_flags(void);

/* Number of launch shapes: integrate_variant takes 0 .. *integrate - 1 and
 * mc_variant 0 .. *mc - 1 (either pointer may be NULL).  Host only. */
void vh_tuning_variants(int32_t *integrate, int32_t *mc);
/* Times every candidate configuration on one frame in a scratch volume with
 * the handle's parameters (the handle's volume is not touched), applies the
 * fastest and returns it in `chosen` (may be NULL).  Results are cached per
 * process and, when the environment variable VHSDF_TUNING_CACHE names a
 * file, in that file, keyed by GPU, image size and volume parameters. */
vh_status vh_autotune(vh_handle *h, const void *depth, int32_t depth_fmt, const uint8_t *rgb,
                      const float *c2w, int32_t mem, vh_tuning *chosen);

/* Decodes a grayscale PNG depth image (8- or 16-bit samples, not
 * interlaced; 16-bit is the millimetre format the reference reads with
 * cv::imread(path, -1) before scaling to metres, src/SaveFrame.cpp:174-180)
 * into out[height * width] uint16, row-major, ready for vh_integrate as
 * VH_DEPTH_U16_MM.  out == NULL: *width and *height only.  Chunk CRCs and
 * the zlib Adler-32 are checked; a malformed stream gives
 * VH_ERR_INVALID_ARG, another colour type, bit depth or interlacing
 * VH_ERR_UNSUPPORTED, capacity < width * height VH_ERR_CAPACITY (the size
 * is reported anyway).  Images up to 2^26 pixels.  Host only. */
vh_status vh_decode_depth_png(const uint8_t *png, int64_t bytes, uint16_t *out,
                              int64_t capacity, int32_t *width, int32_t *height);

/* Decodes a PNG colour frame (RGB, RGBA, grayscale or grayscale + alpha;
 * 8- or 16-bit samples; not interlaced) into rgb[height * width * 3]
 * interleaved R, G, B bytes, row-major: the colour image vh_integrate takes.
 * It stands in for the reference's cv::imread(path, IMREAD_COLOR) followed
 * by its BGR-to-RGB swap (src/SaveFrame.cpp:164, src/main.cpp:273): 16-bit
 * samples keep their high byte, grayscale fills all three channels, alpha is
 * dropped.  rgb == NULL: *width and *height only.  Errors as for
 * vh_decode_depth_png (palette images and bit depths below 8:
 * VH_ERR_UNSUPPORTED; capacity, in bytes, < 3 * width * height:
 * VH_ERR_CAPACITY).  Host only. */
vh_status vh_decode_colour_png(const uint8_t *png, int64_t bytes, uint8_t *rgb,
                               int64_t capacity, int32_t *width, int32_t *height);

/* Decodes a JPEG colour frame, the <i>.jpg files the reference loads with
 * cv::imread(path, IMREAD_COLOR) and swaps to RGB (src/SaveFrame.cpp:164,
 * src/main.cpp:273), into rgb[height * width * 3] interleaved R, G, B
 * bytes.  Sequential Huffman-coded files (baseline and extended, 8-bit
 * samples, grayscale or YCbCr/RGB, any whole chroma subsampling ratio,
 * restart intervals); the exact inverse DCT, a triangle filter for 2x
 * chroma and the JFIF colour transform, so libjpeg's integer arithmetic
 * may differ by one level on some pixels.  An Exif Orientation tag (in an
 * APP1 segment before the frame header) turns or mirrors the image into
 * its displayed orientation, as cv::imread does for IMREAD_COLOR; width
 * and height are then those of the displayed image.  rgb == NULL: *width
 * and *height only.  A malformed stream gives VH_ERR_INVALID_ARG; progressive,
 * lossless, arithmetic-coded, 12-bit and CMYK files VH_ERR_UNSUPPORTED;
 * capacity, in bytes, < 3 * width * height VH_ERR_CAPACITY.  Images up to
 * 2^26 pixels.  Host only. */
vh_status vh_decode_colour_jpeg(const uint8_t *jpg, int64_t bytes, uint8_t *rgb,
                                int64_t capacity, int32_t *width, int32_t *height);

/* Resizes an interleaved RGB u8 image (src_height x src_width x 3) to
 * dst_height x dst_width x 3 by bilinear interpolation, the way the
 * reference brings every colour frame to the depth frame's 640 x 480 grid
 * with cv::resize (src/SaveFrame.cpp:164-171): pixel centres at
 * half-integer positions, sources clamped at the borders, weights in double
 * rounded to the nearest level (OpenCV's fixed-point weights may differ by
 * one level on some pixels).  Sizes 1 .. 32768 per side.  Host only. */
vh_status vh_resize_colour(const uint8_t *src, int32_t src_width, int32_t src_height,
                           uint8_t *dst, int32_t dst_width, int32_t dst_height);

/* Reads frame `frame_id` of a sequence stored in the reference's folder
 * layout (SaveFrame::frameLoad, src/SaveFrame.cpp:44-52,154-218):
 * <root>/depth/<id>.png (16-bit millimetres) into depth[height * width]
 * uint16, <root>/RGB/<id>.jpg or, failing that, <id>.png (decoded by
 * content, JPEG or PNG) into rgb[height * width * 3], resized onto the
 * depth grid when its size differs (vh_resize_colour; the reference
 * resizes to 640 x 480, src/SaveFrame.cpp:171), and <root>/tcw/<id>.txt
 * (16 numbers, each read as the nearest float like the reference's
 * operator>>) into c2w[16], row-major camera-to-world with the last row
 * set to 0 0 0 1 (the reference inverts the matrix twice on the way,
 * src/SaveFrame.cpp:206, src/PointCloudGenerator.cpp:140, which returns
 * it up to float rounding).  The result is ready for vh_integrate with
 * VH_DEPTH_U16_MM.  depth == NULL: *width and *height only.  A missing
 * colour, depth or pose file gives VH_ERR_IO (the frame is missing); too
 * small buffers VH_ERR_CAPACITY; a pose with fewer than 16 numbers
 * VH_ERR_INVALID_ARG, a non-finite one VH_ERR_NOT_FINITE; decoder errors
 * as from the decoders.  Host only. */
vh_status vh_load_frame(const char *root, int32_t frame_id, uint16_t *depth,
                        int64_t depth_capacity, uint8_t *rgb, int64_t rgb_capacity, float *c2w,
                        int32_t *width, int32_t *height);

/* The depth pre-filter of VH_FLAG_DEPTH_FILTER applied to one image: an
 * edge-preserving bilateral filter over 5x5 pixels (spatial sigma 2 px,
 * range sigma 5 mm + 1.5e-3 d^2 x 3, neighbours beyond 3 range sigmas or
 * invalid left out); out[H*W] float metres, 0 where the input is invalid.
 * depth and out in `mem`. */
vh_status vh_filter_depth(vh_handle *h, const void *depth, int32_t depth_fmt, float *out,
                          int32_t mem);

/* ---- out-of-core blocks (the reference streams 128^3-voxel chunks between
 * host and device every frame, src/tsdf.cu:118-596; here the volume stays
 * resident and streaming is explicit) ---------------------------------------- */

/* Moves every GPU block whose centre is farther than `radius` metres from
 * centre[3] (world, host) into the handle's host store (pool layout, bit-
 * identical), freeing its pool block; *moved receives the count (may be
 * NULL).  Blocks moved out are not seen by integration, extraction, export
 * or ray casting until they are moved back in; integrating a frame that
 * reaches them first starts them afresh, and the two copies are merged when
 * they meet again (moved in, or moved out once more): per voxel the weighted
 * average of the two partial averages, sdf (a w_a + b w_b) / (w_a + w_b) in
 * fp32 and colour floor((c_a w_a + c_b w_b) / (w_a + w_b)), weights added;
 * a voxel observed by one copy only keeps that copy's values.  Both
 * directions wait for their copies before returning (the handle's stream is
 * synchronised; they do not overlap frames). */
vh_status vh_stream_out(vh_handle *h, const float *centre, float radius, int64_t *moved);
/* Moves every stored block whose centre is within `radius` of centre[3]
 * back into the volume (radius = INFINITY: all of them): a block with no
 * resident copy comes back bit-identical, one that a frame re-created is
 * merged as vh_stream_out describes.  The keys join the current block list,
 * as vh_alloc_keys does. */
vh_status vh_stream_in(vh_handle *h, const float *centre, float radius, int64_t *moved);
/* vh_stream_out without waiting: the chunk streaming of processFrame
 * (src/tsdf.cu:469-596) done as an eviction that overlaps later frames.  On
 * the handle's stream, in order with the frames around the call, every GPU
 * block whose centre is farther than `radius` metres from centre[3] (at most
 * 32768 per call; the rest stay and a later call takes them) is gathered
 * into a device staging buffer, its key leaves the hash table and its pool
 * block is zeroed and returned to the free list, so frames enqueued after
 * the call neither see the block nor lack its pool space.  A copy kernel on
 * a separate stream then brings the gathered blocks into mapped pinned host
 * memory while those frames run, and the blocks join the host store when a
 * later call finds that copy finished (vh_host_blocks counts them then;
 * vh_sync, vh_stream_in and vh_stream_out wait for it).  Stored copies are
 * bit-identical and merge with re-created blocks as vh_stream_out
 * describes.  Two evictions can be in flight; a third call waits for the
 * older one.  The first call allocates two 192 MiB device staging buffers
 * and two as large in pinned host memory. */
vh_status vh_evict_async(vh_handle *h, const float *centre, float radius);
/* Blocks currently in the host store (evictions whose copy has finished). */
int64_t vh_host_blocks(const vh_handle *h);
/* Rebuilds the hash table from the pool's live blocks, dropping the
 * tombstones that erased keys leave (inserts do not reuse them); the
 * current block list is emptied.  vh_stream_out calls it once tombstones
 * fill an eighth of the table. */
vh_status vh_compact_table(vh_handle *h);

/* ---- ray casting (no reference counterpart: the reference draws its mesh
 * with OpenGL, src/tsdf.cu:1710-1758) ---------------------------------------- */

/* Ray-casts the fused surface from camera pose c2w (row-major 4x4, host)
 * with the handle's image size and intrinsics: depth[H*W] (camera z in
 * metres, 0 where the ray misses), and if not NULL normal[H*W*3] (unit TSDF
 * gradient at the hit, world frame, towards free space) and rgb[H*W*3] (the
 * nearest voxel's colour).  A ray advances by T through unknown space, by
 * 0.8 of the sampled distance (at least half a voxel) through known positive
 * space and by half a voxel through negative space not entered from positive
 * space; the first + -> - change is interpolated linearly.  Outputs in
 * `mem`. */
vh_status vh_raycast(vh_handle *h, const float *c2w, float *depth, float *normal, uint8_t *rgb,
                     int32_t mem);

/* ---- batches of independent scenes (no reference counterpart: the
 * reference runs one scene per process) ------------------------------------ */

typedef struct vh_batch vh_batch;

#define VH_BATCH_MAX_SCENES 1024

/* n independent scenes (1..VH_BATCH_MAX_SCENES) on params[0].device; scene i
 * has params[i]: image size, intrinsics, voxel size, truncation, table and
 * pool sizes may all differ (VH_FLAG_DEPTH_FILTER is not supported in a
 * batch: VH_ERR_UNSUPPORTED).  Every scene is a full handle (vh_batch_scene).
 * The scenes form up to 16 groups of about equal pixel count; each group has
 * its own stream, which is also the stream of its scenes' handles, so calls
 * on a scene handle are ordered with that scene's steps, and groups move
 * from step to step independently (vh_batch_sync joins them).  The launch
 * shapes follow the first scene's tuning (vh_set_tuning / vh_autotune on
 * vh_batch_scene(b, 0)). */
/* With VH_FLAG_BATCH_FUSED in params[0].flags the scenes form one group and
 * a step is one persistent launch (after a one-CTA begin kernel): its CTAs
 * take work items - 2048 pixels of allocation, 256 list entries of resolve,
 * 16 blocks of integration, 4 blocks of marching cubes - from whichever
 * scene has some in its current stage, and the CTA that finishes a scene's
 * stage opens its next one, so one scene's allocation overlaps another's
 * integration inside the launch.  Results are the same either way; the
 * launch shapes then come from that kernel's occupancy, not the tuning. */
vh_status vh_batch_create(const vh_params *params, int32_t n, vh_batch **out);
vh_status vh_batch_destroy(vh_batch *b);
int32_t vh_batch_size(const vh_batch *b);
/* Scene i as an ordinary handle (extract, export, save, stats, hash calls),
 * owned by the batch; NULL if i is out of range. */
vh_handle *vh_batch_scene(vh_batch *b, int32_t i);
/* One frame for every scene i with depth[i] != NULL (the other scenes keep
 * their state): allocation, integration and, with with_mesh, the
 * marching cubes of the frame's blocks.  Each stage is ONE launch per group
 * over the work of all its scenes (flattened scene x item index), and a
 * group's stages of a step replay as one CUDA graph on the group's stream.
 * depth[i] (format depth_fmt, shared) and
 * rgb[i] are in `mem`: host frames are copied into the scene's staging
 * buffers, device frames are read in place by the step (leave them unchanged
 * until it completes); c2w holds n row-major 4x4 poses (host; entries of
 * scenes without a frame are ignored).  Asynchronous unless params[0].flags
 * has VH_FLAG_SYNC, which waits and returns the first scene error (without
 * clearing it); per-scene errors are reported by vh_batch_sync. */
vh_status vh_batch_process(vh_batch *b, const void *const *depth, int32_t depth_fmt,
                           const uint8_t *const *rgb, const float *c2w, int32_t mem,
                           int32_t with_mesh);
/* Waits for the batch; status[i] (may be NULL) receives scene i's sticky
 * device errors as a status (then cleared); stats[i] (may be NULL) its
 * counters after the last step.  One device gather for all scenes.  Returns
 * the first non-OK scene status. */
vh_status vh_batch_sync(vh_batch *b, vh_status *status, vh_stats *stats);

/* ---- gradients and pose refinement (no reference counterpart: the
 * reference has no derivatives) ------------------------------------------- */

#define VH_REFINE_ADJOINT 0 /* analytic Jacobians from the sampling adjoint    */
#define VH_REFINE_FD 1      /* forward-only central differences (13 residual   */
                            /* evaluations per Gauss-Newton step)              */

typedef struct vh_refine_stats {
  int32_t iterations;    /* Gauss-Newton steps taken                         */
  int32_t valid_pixels;  /* residuals in the last linearisation              */
  float initial_rmse;    /* metres, at the initial pose                      */
  float final_rmse;      /* metres, at the last linearised pose              */
  float ms;              /* whole call: depth staging, pose upload, steps,   */
                         /* result download                                  */
  float ms_steps;        /* the Gauss-Newton steps alone (device events)     */
} vh_refine_stats;

/* Trilinear TSDF value (units of the truncation distance) at n world points
 * (x, y, z in metres) and, if grad != NULL, its gradient d sdf / d point
 * (per metre): the adjoint of sampling.  valid[i] = 0 where a corner voxel
 * is unallocated or unobserved (phi and grad are then 0).  All arrays in
 * `mem`. */
vh_status vh_sdf_sample(vh_handle *h, const float *xyz, int64_t n, float *phi, float *grad,
                        uint8_t *valid, int32_t mem);
/* Gauss-Newton normal equations of the SDF residuals r = T * sdf(c2w * X_p)
 * of every `stride`-th pixel of a depth image (truncated samples skipped),
 * for the left perturbation c2w -> exp(xi) c2w, xi = (v, w).  terms[29]:
 * the upper triangle of J^T J row by row (21), J^T r (6), sum r^2, count. */
vh_status vh_pose_normal_equations(vh_handle *h, const void *depth, int32_t depth_fmt,
                                   int32_t mem, const float *c2w, int32_t stride,
                                   int32_t method, double *terms);
/* `iterations` Gauss-Newton steps from c2w_init against the fused volume;
 * writes the refined pose to c2w_out (both row-major 4x4, host).  The steps
 * run on the device without host round trips: each is one kernel launch
 * whose last CTA solves the 6x6 system in FP64 and composes the pose (the
 * launches of a call are replayed as one CUDA graph).  A step whose system is
 * singular or has fewer than 6 residuals ends the refinement early. */
vh_status vh_pose_refine(vh_handle *h, const void *depth, int32_t depth_fmt, int32_t mem,
                         const float *c2w_init, int32_t iterations, int32_t stride,
                         int32_t method, float *c2w_out, vh_refine_stats *stats);
/* Batched refinement (keyframe windows): n poses, each against its own depth
 * image (depth[i], all in `mem` and one format), refined together by the
 * adjoint method - one launch per Gauss-Newton step for all n, the GPU's
 * CTAs split evenly among them, each pose solved by its own last CTA.
 * c2w_init / c2w_out: n * 16 floats (host); stats: n entries or NULL (ms and
 * ms_steps are the whole batch's).  With n = 1 the result equals
 * vh_pose_refine(..., VH_REFINE_ADJOINT, ...) bit for bit. */
#define VH_REFINE_BATCH_MAX 256
vh_status vh_pose_refine_batch(vh_handle *h, const void *const *depth, int32_t depth_fmt,
                               int32_t mem, int32_t n, const float *c2w_init, int32_t iterations,
                               int32_t stride, float *c2w_out, vh_refine_stats *stats);
/* Vector-Jacobian product of the last integration update (depth image and
 * pose c2w of that frame): given dL/dsdf for every voxel of the frame's
 * block list (vh_block_list order, 512 values per block, index x + 8y +
 * 64z), writes dL/ddepth per pixel (H*W floats, metres) and dL/dxi (6
 * floats, host) for the left pose perturbation.  Recomputed from the volume;
 * no per-frame state is kept.  grad_sdf, grad_depth and depth in `mem`. */
vh_status vh_integrate_vjp(vh_handle *h, const void *depth, int32_t depth_fmt, const float *c2w,
                           const float *grad_sdf, float *grad_depth, float *grad_pose,
                           int32_t mem);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* VHSDF_H */
