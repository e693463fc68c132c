/* vdb_gb300.h — C ABI of the GB300 scan-insertion library (libvdb_gb300.so).
 *
 * The reference (vdb_mapping) is a header-only C++ class template with no C
 * ABI; this interface is the boundary its C++ API (the vdb_mapping/ headers
 * in this repository) and any FFI binding call into. Plain pointers, sizes
 * and int status codes only; no exceptions cross it. Every entry point names
 * the reference member it replaces (paths relative to the vdb_mapping tree).
 *
 * Threading: one map may be used from one host thread at a time. All calls
 * that launch GPU work are synchronous unless stated otherwise: they return
 * after the work on the map's stream has completed.
 */
#ifndef VDB_GB300_H
#define VDB_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vdbg_map vdbg_map;

/* Status codes. 1-5 mirror the reference's print-and-return paths. */
enum vdbg_status
{
  VDBG_OK                   = 0,
  VDBG_ERR_NOT_CONFIGURED   = 1,  /* raycast before setConfig (VDBMapping.hpp:478-482) */
  VDBG_ERR_UNKNOWN_SOURCE   = 2,  /* source id not registered (VDBMapping.hpp:321-325) */
  VDBG_ERR_BAD_RANGE        = 3,  /* negative max_range (VDBMapping.hpp:1458-1463) */
  VDBG_ERR_BAD_PROBABILITY  = 4,  /* prob_miss > 0.5 or prob_hit < 0.5 (OccupancyVDBMapping.hpp:65-76) */
  VDBG_ERR_DUPLICATE_SOURCE = 5,  /* source id registered twice */
  VDBG_ERR_INVALID_ARGUMENT = 6,
  VDBG_ERR_OUT_OF_MEMORY    = 7,  /* device allocation failed or memory budget reached */
  VDBG_ERR_COORD_RANGE      = 8,  /* a voxel index outside [-2^21, 2^21) on some axis */
  VDBG_ERR_CUDA             = 9,
  VDBG_ERR_TIMEOUT          = 10, /* a bounded device wait gave up */
  VDBG_ERR_BUFFER_TOO_SMALL = 11,
  VDBG_ERR_SIZE_LIMIT       = 12, /* input larger than a fixed-size entry point accepts */
  VDBG_ERR_BUSY             = 13  /* a serving queue is full; submit again later */
};

/* Input flags. */
#define VDBG_POINTS_DEVICE 1u /* xyz points to device memory (default: host memory) */

/* vdb_mapping::Config (OccupancyVDBMapping.hpp:38-44) with its BaseConfig
 * (VDBMapping.hpp:64-71); map_directory_path is not part of the path. */
typedef struct vdbg_config
{
  double max_range;
  int32_t fast_mode;  /* castRayIntoGridFast (VDBMapping.hpp:577-602): single maps only;
                         vdbg_batch_set_config and the no-allocation insert reject it */
  int32_t reserved0;
  double accumulation_period;
  double prob_hit;
  double prob_miss;
  double prob_thres_min;
  double prob_thres_max;
} vdbg_config;

/* Map creation options (no counterpart in the reference). Zero fields take
 * defaults. */
typedef struct vdbg_options
{
  int64_t initial_leaf_capacity; /* leaf pool slots to reserve (default 65536) */
  int64_t max_device_bytes;      /* growth budget for this map (0 = unlimited) */
  int32_t device;                /* CUDA device ordinal (default current) */
  int32_t initial_block_capacity; /* 64^3-voxel blocks to reserve (default: leaf capacity / 32, >= 1024) */
} vdbg_options;

/* Counters of one call (accumulate, integrate or insert). */
typedef struct vdbg_scan_stats
{
  uint64_t rays;           /* points cast (NaN points are skipped) */
  uint64_t visits;         /* DDA voxel visits plus endpoint hit marks */
  uint64_t hits;           /* unclipped endpoints */
  uint64_t updates;        /* update-grid voxels applied to the map (updateMap iterations) */
  uint64_t new_leaves;     /* 8^3 map leaves created */
  uint64_t touched_leaves; /* leaves swept by the integration */
  uint64_t skipped_nonfinite; /* +-inf points skipped (undefined in the reference) */
  double device_ms;        /* device time of the call's kernels */
} vdbg_scan_stats;

/* VDBMapping(double resolution) VDBMapping.hpp:115-134 / OccupancyVDBMapping.hpp:49. */
int vdbg_create(double resolution, const vdbg_options* options, vdbg_map** out);

/* ~VDBMapping VDBMapping.hpp:139-154. */
int vdbg_destroy(vdbg_map* map);

/* OccupancyVDBMapping::setConfig OccupancyVDBMapping.hpp:59-89 over
 * VDBMapping::setConfig VDBMapping.hpp:1456-1469. Returns BAD_RANGE (nothing
 * changed) or BAD_PROBABILITY (range applied, log-odds kept) like the
 * reference's early returns. */
int vdbg_set_config(vdbg_map* map, const vdbg_config* config);

/* Log-odds constants in use: hit, miss, thres_min, thres_max, max, min. */
int vdbg_get_log_odds(const vdbg_map* map, float out6[6]);

/* VDBMapping::addInputSource VDBMapping.hpp:1352-1375 (max_range 0 selects
 * the configured max_range; no worker thread is started). */
int vdbg_add_input_source(vdbg_map* map, const char* source_id, double max_range, double max_rate);

/* VDBMapping::insertPointCloud VDBMapping.hpp:399-406: accumulate this cloud
 * into the source's update grid, then integrate every source. `xyz` holds n
 * points of three floats at `stride_bytes` spacing (16 for pcl::PointXYZ).
 * An unknown source or missing config returns its status after still running
 * the integration, as the reference does. `stream` is a cudaStream_t or NULL
 * for the map's own stream. */
int vdbg_insert_point_cloud(vdbg_map* map, const float* xyz, int64_t n, int64_t stride_bytes,
                            const double origin[3], const char* source_id, uint32_t flags,
                            void* stream, vdbg_scan_stats* stats);

/* VDBMapping::accumulateUpdate VDBMapping.hpp:316-346. */
int vdbg_accumulate_update(vdbg_map* map, const float* xyz, int64_t n, int64_t stride_bytes,
                           const double origin[3], const char* source_id, uint32_t flags,
                           void* stream, vdbg_scan_stats* stats);

/* VDBMapping::integrateUpdate VDBMapping.hpp:375-387: every source's update
 * grid, in source-id order, then fresh update grids. */
int vdbg_integrate_update(vdbg_map* map, void* stream, vdbg_scan_stats* stats);

/* VDBMapping::raycastPointCloud VDBMapping.hpp:466-539 into the update grid
 * of `source_id` with an explicit raycast range (fast mode as configured). */
int vdbg_raycast_point_cloud(vdbg_map* map, const float* xyz, int64_t n, int64_t stride_bytes,
                             const double origin[3], double raycast_range, const char* source_id,
                             uint32_t flags, void* stream, vdbg_scan_stats* stats);

/* VDBMapping::updateMap VDBMapping.hpp:731-792 for one source's update grid,
 * which is then emptied. */
int vdbg_update_map(vdbg_map* map, const char* source_id, void* stream, vdbg_scan_stats* stats);

/* VDBMapping::resetMap VDBMapping.hpp:174-186. */
int vdbg_reset_map(vdbg_map* map);

/* Number of 8^3 leaves in the map (VDBMapping::getGrid()->tree().leafCount()). */
int vdbg_leaf_count(vdbg_map* map, int64_t* out);

/* VDBMapping::getGrid VDBMapping.hpp:799, as an export: the map's leaves
 * sorted by origin (x, then y, then z). origins: int32[capacity][3] leaf
 * origins (multiples of 8); values: float[capacity][512] log-odds in OpenVDB
 * leaf order (offset = (x&7)<<6 | (y&7)<<3 | (z&7)); masks: uint64[capacity][8]
 * value (active) masks, bit i of word w = voxel offset 64*w+i. Any of the
 * three may be NULL. Returns BUFFER_TOO_SMALL (and the needed count in
 * *n_out) if capacity is too small. */
int vdbg_export_leaves(vdbg_map* map, int64_t capacity, int32_t* origins, float* values,
                       uint64_t* masks, int64_t* n_out);

/* Device-side timing of the last call (no counterpart in the reference),
 * from CUDA events recorded on the call's stream between its kernels. */
typedef struct vdbg_timings
{
  double prep_ms;   /* clip + quantise + L1 bucket sort of the rays */
  double dda_ms;    /* DDA traversal and update-mask marking */
  double sweep_ms;  /* log-odds sweep over the touched leaves */
  double total_ms;  /* first to last kernel of the call */
  uint64_t launches;       /* kernels launched by the call */
  uint64_t launches_total; /* kernels launched by this map since creation */
  uint64_t retries;        /* re-marking passes after a pool or hash growth */
  double apply_ms;         /* the run-merging kernel (k_apply_runs) alone, all passes (part of dda_ms) */
  uint64_t runs;           /* slab runs the traversal wrote (the merging kernel's input) */
  uint64_t passes;         /* DDA passes of the call (more than one when the run buffer filled) */
} vdbg_timings;

int vdbg_get_timings(const vdbg_map* map, vdbg_timings* out);

/* Device bytes held by the map. */
int vdbg_device_bytes(const vdbg_map* map, int64_t* out);

/* The map's pools (no counterpart in the reference, whose OpenVDB tree
 * allocates node by node). Leaf and block slots live in address ranges
 * reserved when the map is created and are backed by device memory as they
 * are needed, so a slot never moves and growing a pool copies nothing. While
 * a call's kernels run, the library backs and initialises the next stretch
 * of slots when the pool is about to run short ("ahead"); a call that still
 * runs out grows the pool on the spot ("sync") and retries its marking. */
typedef struct vdbg_pool_info
{
  int64_t leaf_capacity;   /* leaf slots the kernels may use */
  int64_t leaf_backed;     /* leaf slots backed and initialised (>= leaf_capacity) */
  int64_t leaf_reserved;   /* leaf slots the address range can hold */
  int64_t leaves;          /* leaves in use */
  int64_t block_capacity;  /* 64^3-voxel block slots the kernels may use */
  int64_t blocks;          /* blocks in use */
  int64_t hash_entries;    /* block hash size */
  uint64_t grow_ahead;     /* extensions prepared while kernels ran */
  uint64_t grow_sync;      /* extensions made because a call ran out */
} vdbg_pool_info;

int vdbg_get_pool_info(const vdbg_map* map, vdbg_pool_info* out);

/* Verification digests (no counterpart in the reference): numbers that
 * summarise a traversal or a map exactly, for comparisons at sizes where
 * exporting everything is impractical (the oracle computes the same).
 *
 * vdbg_ray_digests: castRayIntoGrid (VDBMapping.hpp:550-566) of every point
 * of the cloud, as raycastPointCloud (VDBMapping.hpp:499-530) sets it up for
 * this map with `raycast_range`, walked by the insertion's own DDA but marking
 * nothing. out: uint64[n][2], per point: word 0 = visited voxels | clipped <<
 * 40 | valid << 41 (NaN and infinite points are not valid), word 1 = a hash
 * chain over the visited voxels in order and the end voxel:
 *   k(x,y,z) = u32(x)*0x9E3779B97F4A7C15 ^ u32(y)*0xC2B2AE3D27D4EB4F
 *              ^ u32(z)*0x165667B19E3779F9
 *   h = 0x243F6A8885A308D3; h = fmix64(h ^ k(v)) per visited voxel v;
 *   h = fmix64(h ^ k(end) ^ 0x5851F42D4C957F2D)
 * (fmix64: MurmurHash3's 64-bit finaliser). The map is not changed.
 *
 * vdbg_map_digest: out[4] = {leaves, voxels, leaf sum, voxel sum} of map
 * `map_index` (-1: every map of a batch), the sums mod 2^64 of fmix64(k(leaf
 * origin)) over its leaves and of fmix64(k(x,y,z) ^ (bits << 1 | active) *
 * 0xD6E8FEB86659FD93) over its voxels whose FP32 value bits are non-zero or
 * that are active. */
int vdbg_ray_digests(vdbg_map* map, const float* xyz, int64_t n, int64_t stride_bytes, const double origin[3],
                     double raycast_range, uint32_t flags, uint64_t* out);
int vdbg_map_digest(vdbg_map* map, int map_index, uint64_t out[4]);

/* L2 atomic throughput of `device` (no counterpart in the reference): the
 * rate of 64-bit ORs with unused results (reductions) on an L2-resident
 * buffer, in operations per second, best of three timed launches. pattern 0:
 * a warp ORs 32 consecutive words per request (the shape of the update-mask
 * merges); 1: every lane a pseudo-random word (the endpoint hits). It is the
 * denominator of the atomic half of the insertion's roofline. */
int vdbg_l2_atomic_rate(int device, int pattern, double* ops_per_s);

/* Change set (the grid updateMap returns, VDBMapping.hpp:731-792): with
 * tracking on, every call that integrates (insert, integrate_update,
 * update_map, batch insert) replaces the change set with the voxels whose
 * active state its update grid flipped: `active` holds the flipped voxels,
 * `value` those flipped on (by a hit); a miss only turns voxels off. When a
 * call integrates several sources' update grids the set is that of the last
 * one (sources integrate in id order). vdbg_export_changes returns the leaves
 * with a flip, sorted by origin: origins int32[n][3], active and value
 * uint64[n][8] (bit i of word w = leaf offset 64w+i), of map `map` of a batch
 * (-1: every map). Tracking costs 136 bytes per leaf slot and a little sweep
 * time; off by default. */
int vdbg_track_changes(vdbg_map* map, int enable);
int vdbg_export_changes(vdbg_map* map, int map_index, int64_t capacity, int32_t* origins, uint64_t* active,
                        uint64_t* value, int64_t* n_out);

/* Launch and layout parameters of the insertion kernels (no counterpart in
 * the reference). They change speed only, never results; the package's
 * autotuner (vdb_mapping_gb300/autotune.py) picks them by timing candidates
 * on a sample of the caller's scans. */
typedef struct vdbg_tuning
{
  int32_t rays_per_take;     /* rays a DDA warp takes from the sorted order at a time (1-1024; 32) */
  int32_t apply_chunk_runs;  /* DDA runs an apply block stages and merges at a time (256-4096, a multiple of 256; 2048) */
  int32_t length_edges[3];   /* L1 lengths (voxels) starting the sort's length classes, descending (2048, 1024, 512) */
  float hash_load;           /* block-hash load factor (0.05-0.9; 0.5); a change rebuilds the hash */
  int32_t dda_warps_per_sm;  /* resident DDA warps per SM (2-20, even; 16) */
  int32_t sweep_kernel;      /* 0 (default): one z-plane per lane, or for a batch of maps eight lanes
                                per z-plane when its previous sweep updated 16-30 voxels per touched
                                leaf; 1: one z-plane per lane; 2: eight lanes per z-plane */
} vdbg_tuning;

int vdbg_set_tuning(vdbg_map* map, const vdbg_tuning* tuning);
int vdbg_get_tuning(const vdbg_map* map, vdbg_tuning* out);

/* Insertion that allocates no device memory during the call. No counterpart
 * in the reference: it exists for callers that must not allocate while they
 * run, such as real-time mapping loops where cudaMalloc's unbounded latency
 * and implicit device synchronisation break the cycle budget, or hosts that
 * own all device memory through their own pool. Same semantics and results as
 * vdbg_insert_point_cloud, but the per-scan scratch lives in one fixed
 * VDBG_NOALLOC_SCRATCH_BYTES device array inside the library (held by every
 * GPU that loads it, until the process exits) instead of buffers the map
 * grows on demand. It also runs its ray traversal on fewer warps, in as many
 * passes as the scan needs, so it is slower than the regular call. Limits:
 * n <= VDBG_NOALLOC_MAX_POINTS and, for host input,
 * stride_bytes <= 16; larger inputs return VDBG_ERR_SIZE_LIMIT. The map's leaf
 * pool is not grown: when it is full the call returns VDBG_ERR_OUT_OF_MEMORY,
 * applies nothing and discards the source's pending update grid, so create
 * the map with an initial_leaf_capacity that covers its extent. The first
 * call on a device looks up the array's device address (a one-time set-up);
 * make that first call before any stream capture. All calls share the array,
 * so calls that overlap on the GPU (other threads, other streams, other maps)
 * race: serialise them. */
#define VDBG_NOALLOC_MAX_POINTS 262144
#define VDBG_NOALLOC_DDA_WARPS 256
#define VDBG_NOALLOC_RUN_SEGMENT 4096
#define VDBG_NOALLOC_SCRATCH_BYTES (28u << 20)
int vdbg_insert_point_cloud_noalloc(vdbg_map* map, const float* xyz, int64_t n, int64_t stride_bytes,
                                    const double origin[3], const char* source_id, uint32_t flags,
                                    void* stream, vdbg_scan_stats* stats);

/* Batches of independent maps. No counterpart in the reference, which runs
 * one OccupancyVDBMapping per map: here up to 126 maps with their own
 * resolutions and configs share one device pool, and one call inserts one
 * scan into each map (insertPointCloud, VDBMapping.hpp:399-406, for every map
 * at once) through a single pass of the kernels. Each map's result equals
 * what inserting its scan alone into its own map would give. The single-map
 * entry points reject batch handles; vdbg_destroy, vdbg_reset_map,
 * vdbg_leaf_count (all maps), vdbg_get_timings and vdbg_device_bytes accept
 * them. */
int vdbg_create_batch(int n_maps, const double* resolutions, const vdbg_options* options, vdbg_map** out);

/* setConfig (OccupancyVDBMapping.hpp:59-89) of map `map` of a batch; a map's
 * scans are cast to its max_range (0: that map's scans are not cast). */
int vdbg_batch_set_config(vdbg_map* batch, int map, const vdbg_config* config);

/* One scan per map: counts[i] points of map i, concatenated in map order in
 * xyz (stride_bytes apart), origins[3*i..3*i+2] its sensor origin. Maps with
 * no points, a zero max_range or a NaN origin are skipped. A voxel index out
 * of range in any scan leaves every map of the batch unchanged and returns
 * VDBG_ERR_COORD_RANGE. stats receives the totals over the batch. */
int vdbg_batch_insert(vdbg_map* batch, const float* xyz, const int64_t* counts, int64_t stride_bytes,
                      const double* origins, uint32_t flags, void* stream, vdbg_scan_stats* stats);

/* Map sections. `map` is -1 (or 0) for a single-map handle, the map's index
 * for a batch. Boxes are index boxes [lo, hi], inclusive: the reference
 * builds them with createIndexBoundingBox (VDBMapping.hpp:858-870) from a world
 * box and a transform; the C++ drop-in and the Python package provide that
 * step. Leaves are in vdbg_export_leaves' layout, sorted by origin.
 *
 * getMapSectionGrid / getMapSectionUpdateGrid (VDBMapping.hpp:883-962): the
 * map's leaves overlapping the box, restricted to the voxels inside it.
 * full != 0 keeps each inside voxel's value and state (extractFullLeaf,
 * :972-990). full == 0 gives the active inside voxels value 1 (extractSparseLeaf,
 * :1001-1012; an update grid reads the values as bool). The others are the
 * background 0, inactive. A leaf is returned only if a write created it: it
 * holds an active inside voxel or, full, an inside value other than 0. */
int vdbg_export_section(vdbg_map* map, int map_index, const int32_t lo[3], const int32_t hi[3], int full,
                        int64_t capacity, int32_t* origins, float* values, uint64_t* masks, int64_t* n_out);

/* applyMapSectionUpdateGrid (VDBMapping.hpp:1058-1085): every active map
 * voxel inside [lo, hi] (the section's bb_min/bb_max) is set inactive, then
 * every active voxel of the n section leaves is set active. Values are kept,
 * and a new leaf starts at 0. With smoothing, the caller closes the section
 * first with vdbg_section_morphology (op 2). */
int vdbg_apply_section_states(vdbg_map* map, int map_index, const int32_t lo[3], const int32_t hi[3], int64_t n,
                              const int32_t* origins, const uint64_t* masks);

/* applyMapSectionGrid without smoothing (VDBMapping.hpp:1022-1048). Each
 * section leaf's 512 values and states overwrite the map leaf, which is
 * created unless every voxel is inactive 0. The section tree's tiles, the
 * empty slots of its 128^3 and 4096^3 internal nodes, set the map voxel at
 * their origin to inactive 0 where a map leaf holds it, as the reference's
 * cbeginValueAll() does. Smoothing (morphologicalCloseMap, :1026-1029) is
 * vdbg_section_morphology with VDBG_MORPH_KEEP_LEAVES first. */
int vdbg_apply_section_values(vdbg_map* map, int map_index, int64_t n, const int32_t* origins, const float* values,
                              const uint64_t* masks);

/* Artificial areas (VDBMapping.hpp:1152-1236), single maps only.
 * vdbg_add_artificial_walls is addArtificialWall (:1210-1236) for n walls
 * (world start and end points [n][3]): both ends go through worldToIndex,
 * and for every layer i in [(int)(negative_height / res),
 * (int)(positive_height / res)) the voxels castRayIntoGrid visits from
 * start + (0,0,i) to end + (0,0,i) join the artificial set. After every
 * update of the map that integrates a non-empty update grid, each artificial
 * voxel is set active, its leaf created at the background when absent
 * (updateMap, :785-789). addArtificialPolygon is the walls between
 * consecutive corners, closing back to the first; addArtificialAreas is
 * vdbg_restore_map_integrity, then its polygons.
 * vdbg_restore_map_integrity is restoreMapIntegrity (:1153-1166): every
 * artificial voxel's state becomes value > the log-odds of prob_thres_max
 * (setNodeState), then the set is emptied. The no-allocation insert rejects
 * a map with artificial areas. */
int vdbg_add_artificial_walls(vdbg_map* map, int64_t n, const double* starts, const double* ends,
                              double negative_height, double positive_height);
int vdbg_restore_map_integrity(vdbg_map* map);

/* Test hook for the bounded device waits (no counterpart in the reference).
 * Leaves the empty cell of leaf (lx, ly, lz) (voxel coordinates / 8) of the
 * map (map_index -1) or map `map_index` of a batch pending, as if a thread
 * had claimed it and never published its slot. The next call whose rays
 * reach that leaf waits for the slot up to the wait's bound (about a
 * second), then returns VDBG_ERR_TIMEOUT with its marking discarded; the
 * map and the context stay usable, and vdbg_reset_map clears the cell.
 * VDBG_ERR_INVALID_ARGUMENT when the leaf exists. */
int vdbg_test_stall_leaf(vdbg_map* map, int map_index, int32_t lx, int32_t ly, int32_t lz);

/* Morphology of a map section's active voxels with the 26-neighbourhood:
 * openvdb::tools::dilateActiveValues / erodeActiveValues with
 * NN_FACE_EDGE_VERTEX as VDBMapping.hpp:1094-1147 calls them
 * (morphologicalDilateMap op 0, ErodeMap 1, CloseMap 2 = dilate then erode,
 * OpenMap 3 = erode then dilate, `iterations` steps each, 0..64). A dilation
 * step activates every voxel with an active voxel among its 26 neighbours, an
 * erosion step keeps the active voxels whose 26 neighbours are all active;
 * voxels outside the leaves are inactive. Input: n leaves (origins multiples
 * of 8 within +-2^20, masks in vdbg_export_leaves' layout; a repeated origin's
 * masks are merged). Output: the leaves holding active voxels, sorted by
 * origin, *n_out of them (VDBG_ERR_BUFFER_TOO_SMALL when capacity is less).
 * Runs on the map's device and stream; the map is not changed.
 * applyMapSectionUpdateGrid's smoothing (VDBMapping.hpp:1062-1065) is op 2
 * before vdbg_apply_section_states.
 * op | VDBG_MORPH_KEEP_LEAVES keeps the leaf topology as OpenVDB's morphology
 * leaves a tree it does not prune: the output holds every input leaf and
 * every leaf a dilation step set bits in, empty or not (erosion removes no
 * leaf). applyMapSectionGrid's smoothing (VDBMapping.hpp:1026-1029) is op 2
 * with this flag; the leaves it adds take the value 0, the others keep
 * theirs, before vdbg_apply_section_values. */
#define VDBG_MORPH_KEEP_LEAVES 16
int vdbg_section_morphology(vdbg_map* map, int op, int iterations, int64_t n, const int32_t* origins,
                            const uint64_t* masks, int64_t capacity, int32_t* out_origins, uint64_t* out_masks,
                            int64_t* n_out);

/* VDBMapping::raytrace VDBMapping.hpp:675-721 (the single-ray overload,
 * :646-662, is n = 1) for the map (map_index -1) or map `map_index` of a
 * batch: n rays with world origins[n][3], directions[n][3] (normalised here)
 * and max_lengths[n]; successes[n] (1 when the volume ray intersector found a
 * span of leaves on the ray) and end_points[n][3] (the first active voxel
 * after the span's start voxel, or the voxel just past the span, or, without
 * a span, the ray's end) out, all in host memory. The intersector is that of
 * fast mode (VDBMapping.hpp:1436-1449) on the map as it stands; the reference
 * has one only in fast mode, this call works in either mode. A ray whose
 * index-space start or end is NaN or outside +-2^30 fails the call with
 * VDBG_ERR_COORD_RANGE. */
int vdbg_raytrace(vdbg_map* map, int map_index, int64_t n, const double* origins, const double* directions,
                  const double* max_lengths, uint8_t* successes, double* end_points);

/* CUDA-graph replay of vdbg_batch_insert (batches of two or more maps; on by
 * default). The step is captured once per buffer layout and replayed as one
 * graph launch: prep, endpoint hits, the first DDA pass with its apply,
 * compact, sweep. It is captured again after a pool, scratch or run-buffer
 * reallocation or a tuning change (the input's address and point counts
 * reach the graph through device memory). When a step
 * needs a second DDA pass or a pool to grow, the graph's compact and sweep
 * skip themselves on the device and the call finishes the step with separate
 * launches. Off, or with change tracking on, every step uses separate
 * launches; the results are the same either way. vdbg_graph_stats reports
 * the captures and replays so far. */
int vdbg_batch_use_graph(vdbg_map* batch, int enable);
int vdbg_graph_stats(const vdbg_map* batch, uint64_t* captures, uint64_t* replays);

/* Leaf count and export (as vdbg_leaf_count / vdbg_export_leaves) of one map. */
int vdbg_batch_leaf_count(vdbg_map* batch, int map, int64_t* out);
int vdbg_batch_export_leaves(vdbg_map* batch, int map, int64_t capacity, int32_t* origins, float* values,
                             uint64_t* masks, int64_t* n_out);

/* Serving loop over a batch (continuous batching). No counterpart in the
 * reference, whose per-source worker threads (VDBMapping.hpp:1383-1430) each
 * feed one map. One worker thread serves every sensor stream of a batch:
 * vdbg_server_submit copies a scan into pinned staging and queues it on its
 * map's FIFO without waiting for the GPU; the worker forms every step from
 * the oldest queued scan of each map (so a map's scans apply in submission
 * order), admits them against memory_budget_bytes (a scan whose map would
 * need the pool to grow past the budget waits for a step of its own, and is
 * completed with VDBG_ERR_OUT_OF_MEMORY if even then it does not fit), and
 * inserts them with one batched call; scans arriving meanwhile join the next
 * step. Steps are pipelined: while the device marks and sweeps one step, the
 * next is formed from what has arrived and its upload and ray preparation run
 * on a second stream beside it; its marking starts when the step before ends.
 * A scan's result is the same whatever it shares a step with. While a
 * server runs, only the server calls may touch its batch; destroy the server
 * before using the batch directly again. */
typedef struct vdbg_server vdbg_server;

typedef struct vdbg_server_options
{
  int64_t memory_budget_bytes; /* device bytes the batch may hold (0: no budget) */
  int32_t max_batch_maps;      /* most maps per step (0: all) */
  int32_t queue_capacity;      /* most queued scans before submit returns VDBG_ERR_BUSY (0: 4096) */
} vdbg_server_options;

typedef struct vdbg_server_result
{
  uint64_t tag;        /* the caller's tag of the request */
  int32_t map;
  int32_t status;      /* VDBG_OK or the batched call's status */
  int64_t points;
  int64_t submit_ns;   /* steady-clock times: queued, step started, step done */
  int64_t start_ns;
  int64_t done_ns;
  int32_t batch_maps;  /* scans in the step that served it */
  int32_t reserved0;
} vdbg_server_result;

typedef struct vdbg_server_stats
{
  int64_t requests_submitted;
  int64_t requests_done;
  int64_t rejected;      /* completed with VDBG_ERR_OUT_OF_MEMORY by admission */
  int64_t steps;
  int64_t max_step_maps;
  int64_t queued;
  int64_t max_queued;
  uint64_t rays;
  uint64_t updates;
  int64_t busy_ns;       /* time spent in batched calls */
  int64_t device_bytes;
  int64_t overlapped_steps; /* steps during which the next step's upload and ray preparation were queued */
} vdbg_server_stats;

int vdbg_server_create(vdbg_map* batch, const vdbg_server_options* options, vdbg_server** out);
/* Queues one scan of map `map` (n points stride_bytes apart, host memory). */
int vdbg_server_submit(vdbg_server* server, int map, const float* xyz, int64_t n, int64_t stride_bytes,
                       const double origin[3], uint64_t tag);
/* Up to `capacity` completed requests, waiting up to wait_ms for the first. */
int vdbg_server_poll(vdbg_server* server, vdbg_server_result* out, int capacity, int wait_ms, int* n_out);
/* Waits (up to wait_ms) until every submitted scan has completed. */
int vdbg_server_drain(vdbg_server* server, int wait_ms);
int vdbg_server_get_stats(vdbg_server* server, vdbg_server_stats* out);
/* Completes the queued scans, stops the worker and frees the server (not the batch). */
int vdbg_server_destroy(vdbg_server* server);

/* Human-readable text of a status code (static storage). */
const char* vdbg_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif /* VDB_GB300_H */
