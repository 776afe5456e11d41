/*
 * OctreeApi -- C ABI of the GB300 LOD octree builder (libOctreeApi.so).
 *
 * Drop-in for the OctreeApi session API of PotreeConverterGPU.  The first 18
 * entry points keep the reference's names, argument meaning, call order and
 * return convention (0 = SUCCESS, -1 = UNEXPECTED_ERROR); each comment cites
 * the reference declaration it replaces (OctreeApi/include/octreeApi.h) and
 * implementation (OctreeApi/src/octreeApi.cpp, OctreeApi/src/session.cpp).
 *
 * Differences a caller can observe:
 *   - CUDA and configuration errors return -1 (the reference calls exit(),
 *     OctreeLibrary/include/defines.cuh:18-30); ocpi_last_error() describes
 *     the last failure of the calling thread.
 *   - Each session has its own device state, stream and statistics; sessions
 *     on different host threads may run concurrently.
 *   - octree.bin holds exactly the records referenced by hierarchy.bin (the
 *     reference writes its whole, partly uninitialised, output buffer).
 * Entry points after the first 18 are additions with no reference
 * counterpart.
 */
#ifndef OCTREE_API_H
#define OCTREE_API_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
#define OCPI_EXPORT extern "C" __attribute__((visibility("default")))
#else
#define OCPI_EXPORT __attribute__((visibility("default")))
#endif

#define SUCCESS (0)
#define UNEXPECTED_ERROR (-1)

/* ---- session: octreeApi.h:42-44, octreeApi.cpp:96-128, session.cpp:87-112 */
OCPI_EXPORT int ocpi_create_session(void** session, int device);
OCPI_EXPORT int ocpi_destroy_session(void* session);
/* 0 debug, 1 info, 2 warn, 3 error (octreeApi.cpp:96-115) */
OCPI_EXPORT int ocpi_set_logging_level(int level);

/* ---- cloud description: octreeApi.h:46-54, session.cpp:115-120,180-208 */
/* 0 = float32 xyz + u8 rgb (15-byte records), 1 = float64 xyz + u8 rgb (27) */
OCPI_EXPORT int ocpi_set_cloud_type(void* session, uint8_t cloudType);
OCPI_EXPORT int ocpi_set_cloud_point_amount(void* session, uint32_t pointAmount);
OCPI_EXPORT int ocpi_set_cloud_data_stride(void* session, uint32_t dataStride);
OCPI_EXPORT int ocpi_set_cloud_scale(void* session, double x, double y, double z);
/* stored only; no stage uses the offset (as in the reference) */
OCPI_EXPORT int ocpi_set_cloud_offset(void* session, double x, double y, double z);
/* the cubic bounding box (src/boundingbox.h:35-52 computes it in the CLI) */
OCPI_EXPORT int ocpi_set_cloud_bb(void* session, double minX, double minY, double minZ, double maxX, double maxY,
                                  double maxZ);
/* borrowed host pointer, read by ocpi_init_octree */
OCPI_EXPORT int ocpi_set_point_cloud_host(void* session, uint8_t* pointCloud);

/* ---- configuration: octreeApi.h:56-65, session.cpp:158-179 */
OCPI_EXPORT int ocpi_configure_chunking(void* session, uint32_t chunkingGrid, uint32_t mergingThreshold,
                                        float outputFactor);
OCPI_EXPORT int ocpi_configure_subsampling(void* session, uint32_t subsamplingGrid, bool intraCellAveraging,
                                           bool interCellAveraging, bool replacementScheme,
                                           bool useRandomSubsampling, bool useWeightingFunction);

/* ---- reports: octreeApi.h:67-69, session.cpp:139-156 */
OCPI_EXPORT int ocpi_export_memory_report(void* session, const char* filename);
OCPI_EXPORT int ocpi_export_distribution_histogram(void* session, const char* filename, uint32_t binWidth);
OCPI_EXPORT int ocpi_export_json_report(void* session, const char* filename);

/* ---- pipeline: octreeApi.h:70-72, session.cpp:62-77,211-214 */
OCPI_EXPORT int ocpi_export_potree(void* session, const char* directory);
/* allocates device memory and uploads the cloud */
OCPI_EXPORT int ocpi_init_octree(void* session);
/* counting, merging, distribution and subsampling */
OCPI_EXPORT int ocpi_generate_octree(void* session);

/* ======================================================================= */
/* Additions (no reference counterpart).                                   */

/* Message of the last failed call on this host thread ("" if none). */
OCPI_EXPORT const char* ocpi_last_error(void);
/* Seed of the explicit-random subsampling priorities (default 0x5EED). */
OCPI_EXPORT int ocpi_set_random_seed(void* session, uint64_t seed);
/* Debug switches: bit 0 keeps a copy of the count pyramid (dense per level,
 * z-major order) for ocpi_get_level_counts. */
OCPI_EXPORT int ocpi_set_debug_flags(void* session, uint32_t flags);

typedef struct OcpiStats {
    uint64_t points_total;   /* records referenced by the hierarchy (N + subsampled) */
    uint64_t p_out;          /* points held by internal nodes */
    uint64_t p_in;           /* candidate points read by subsampling */
    uint64_t out_capacity;   /* the reference's output buffer size for this config */
    uint32_t depth;
    uint32_t tree_nodes;
    uint32_t leaf_nodes;
    uint32_t internal_nodes;
    uint32_t sparse_nodes;   /* occupied cells over all pyramid levels */
    uint32_t dense_nodes;
    uint32_t max_leaf_depth;
    uint32_t min_leaf_points;
    uint32_t max_leaf_points;
    float mean_leaf_points;
    float stdev_leaf_points;
    uint32_t kernel_launches; /* kernels launched by the last ocpi_generate_octree */
    uint32_t subsample_passes; /* subsampling passes of the last build: 1, or more when a level's
                                  candidates or the final records outgrew their buffers and the
                                  pass was repeated with larger ones */
} OcpiStats;

OCPI_EXPORT int ocpi_get_stats(void* session, OcpiStats* out);
/* hierarchy.bin content: node_count entries of 22 bytes, BFS order */
OCPI_EXPORT int ocpi_get_node_count(void* session, uint64_t* count);
OCPI_EXPORT int ocpi_get_hierarchy(void* session, uint8_t* out);
/* octree.bin content: points_total records of 18 bytes, and for each record
 * the index of its source point in the cloud */
OCPI_EXPORT int ocpi_get_records(void* session, uint8_t* out);
OCPI_EXPORT int ocpi_get_lut(void* session, uint32_t* out);
/* dense count grid of one pyramid level (requires debug bit 0) */
OCPI_EXPORT int ocpi_get_level_counts(void* session, uint32_t level, uint32_t* out);
/* Stage timings of the last ocpi_init_octree / ocpi_generate_octree, in ms,
 * measured with CUDA events on the session stream.  Writes up to `max`
 * values and their names (comma separated) into names (size name_bytes). */
OCPI_EXPORT int ocpi_get_timings(void* session, double* ms, int max, char* names, int name_bytes, int* count);

/* Bounding box on the device: calculateRealBB + calculateCubicBB
 * (src/boundingbox.h:11-52, computed on the host by the reference CLI) over
 * the cloud uploaded by ocpi_init_octree, exactly (min / max of the
 * coordinates, NaN skipped, then the reference's cube arithmetic).  The cubic
 * box becomes the session's bounding box, so ocpi_set_cloud_bb may be left
 * out before ocpi_init_octree.  realBB / cubicBB (either may be NULL) receive
 * {minX, minY, minZ, maxX, maxY, maxZ}. */
OCPI_EXPORT int ocpi_compute_cloud_bb(void* session, double* realBB, double* cubicBB);

/* Device memory the session holds now, in bytes (all its allocations). */
OCPI_EXPORT int ocpi_get_device_memory(void* session, uint64_t* bytes);

/* Memory estimate for a configuration, before anything is allocated (e.g. for
 * admission): gb300Bytes is an upper bound of what a session of this library
 * allocates (data-dependent buffers at their capacity rules, valid for every
 * build whose output fits outputFactor * N records); referenceBytes is the
 * reference's estimate (tools/memory_consumption.py:30-75) extended by the
 * sparse node array, per-node counters and the weighted RGBA grid.
 * modeFlags: OCPI_SUB_* bits (defined below).  Needs no GPU. */
OCPI_EXPORT int ocpi_estimate_memory(uint32_t pointAmount, uint32_t dataStride, uint8_t cloudType,
                                     uint32_t chunkingGrid, uint32_t mergingThreshold, float outputFactor,
                                     uint32_t subsamplingGrid, uint32_t modeFlags, uint64_t* gb300Bytes,
                                     uint64_t* referenceBytes);

/* Registers host arrays that every later ocpi_generate_octree fills before it
 * returns: octree.bin records (and, if lut is not NULL, the source index of
 * each record), `capacity` records each.  The leaf records are copied while
 * the upper levels are being subsampled, so with page-locked (pinned) arrays
 * most of the read-back overlaps the build.  ocpi_get_records / ocpi_get_lut
 * on the same arrays then copy nothing.  The arrays must stay valid until the
 * next ocpi_generate_octree returns; generate fails when the octree has more
 * than `capacity` records (outputFactor * N is always enough for builds the
 * reference can hold).  records = NULL unregisters. */
OCPI_EXPORT int ocpi_set_output_host(void* session, uint8_t* records, uint32_t* lut, uint64_t capacity);

/* ---- batched and served forms (no counterpart in the reference) ---------
 *
 * An executor runs independent builds at once on one GPU: `lanes` worker
 * threads, each with its own builder, streams and grow-only buffers (a lane
 * reuses its buffers from job to job, so a warm executor allocates nothing).
 * Admission: a job's device memory is bounded as by ocpi_estimate_memory; a
 * lane reserves the largest bound it has run, and a job starts only while the
 * lanes' reservations fit memoryBudget (oldest fitting job first; an idle
 * lane gives its memory back when a waiting job needs it).  A job whose bound
 * alone exceeds the budget is refused at submission.  Each result equals the
 * same build run alone through the session API. */
typedef struct OcpiJob {
    const uint8_t* cloud;      /* host records; must stay valid until the job completes */
    uint32_t pointAmount;
    uint32_t dataStride;
    uint8_t cloudType;         /* 0 float32, 1 float64 */
    double scale[3];
    double bbMin[3];           /* cubic bounding box; all six zero: computed on the device */
    double bbMax[3];
    uint32_t chunkingGrid;
    uint32_t mergingThreshold;
    float outputFactor;
    uint32_t subsamplingGrid;
    uint32_t modeFlags;        /* OCPI_SUB_* bits */
    uint64_t seed;             /* explicit-random seed */
    uint8_t* outRecords;       /* optional host array for octree.bin (see ocpi_set_output_host) */
    uint32_t* outLut;          /* optional */
    uint64_t outCapacity;      /* records */
    uint8_t* outHierarchy;     /* optional host array for hierarchy.bin */
    uint64_t outHierarchyCapacity;   /* bytes */
    uint64_t cloudId;          /* 0, or an id naming this cloud's contents: a lane that built the same id with the
                                  same chunking settings reruns only subsampling on its resident device state */
} OcpiJob;

typedef struct OcpiJobResult {
    int32_t status;            /* 0 = built, -1 = failed (error holds the message) */
    uint32_t lane;
    uint32_t nodeCount;        /* hierarchy.bin entries */
    uint32_t reused;           /* 1: subsampled the lane's resident cloud state (no upload, counting or distribution) */
    uint64_t pointsTotal;      /* octree.bin records */
    double queuedMs;           /* submission to start */
    double runMs;              /* start to completion (upload, build, read-back) */
    double totalMs;            /* submission to completion */
    double deviceMs;           /* build stages, CUDA events */
    char error[128];
    uint32_t subsamplePasses;  /* as OcpiStats.subsample_passes; a build of a subsampling wave that
                                  outgrew its buffers repeats its pass alone */
} OcpiJobResult;

OCPI_EXPORT int ocpi_server_create(void** server, int device, uint32_t lanes, uint64_t memoryBudget);
/* waits for the jobs in progress */
OCPI_EXPORT int ocpi_server_destroy(void* server);
OCPI_EXPORT int ocpi_server_submit(void* server, const OcpiJob* job, uint64_t* ticket);
/* blocks until the job completes */
OCPI_EXPORT int ocpi_server_wait(void* server, uint64_t ticket, OcpiJobResult* result);
OCPI_EXPORT int ocpi_server_get_hierarchy(void* server, uint64_t ticket, uint8_t* out);
/* forgets a completed job (waits for it first) */
OCPI_EXPORT int ocpi_server_release(void* server, uint64_t ticket);
/* a waiting job completes as failed ("cancelled"): at once when queued, and
   after its lane's current job when a lane already holds it; -1 if it is
   running or done */
OCPI_EXPORT int ocpi_server_cancel(void* server, uint64_t ticket);
/* how many times a lane restarted after losing its worker */
OCPI_EXPORT int ocpi_server_lane_restarts(void* server, uint64_t* restarts);

/* Host-side fault injection for tests (no GPU fault is involved): the next
 * `count` events of a kind fail.  OCPI_INJECT_ALLOCATION: a device or pinned
 * allocation of any session or lane fails as if cudaMalloc had (the call
 * returns -1, the job fails).  OCPI_INJECT_LANE_LOSS: a server lane that takes
 * a job drops it and its state as if its worker had died, then restarts.
 * count 0 clears a kind. */
#define OCPI_INJECT_ALLOCATION 1
#define OCPI_INJECT_LANE_LOSS 2
OCPI_EXPORT int ocpi_debug_inject_failures(int kind, uint32_t count);
/* all jobs submitted at once to an executor that the library keeps for the
 * rest of the process (one per device, lanes and budget), so that its lanes'
 * device buffers stay allocated between batches; returns -1 if any failed */
OCPI_EXPORT int ocpi_batch_build(int device, uint32_t lanes, uint64_t memoryBudget, const OcpiJob* jobs,
                                 uint32_t count, OcpiJobResult* results);
/* the same batch in subsampling waves: jobs grouped by record type and
 * subsampling mode, built waveSize at a time on pooled builders; each wave's
 * subsampling, every level of all its builds with one launch per level, is
 * captured into one CUDA graph.  waveSize 0: the tuning that
 * ocpi_batch_autotune chose for a batch like this one, autotuning on this
 * batch first when there is none */
OCPI_EXPORT int ocpi_batch_build_wave(int device, uint32_t waveSize, uint64_t memoryBudget, const OcpiJob* jobs,
                                      uint32_t count, OcpiJobResult* results);

/* Tuning of the batched form: subsampling waves, or the lane executor. */
typedef struct OcpiBatchTuning {
    uint32_t waveSize;            /* builds per wave, 1..256 */
    uint32_t clusterCap;          /* largest thread-block cluster per node of a subsampling level: 1, 2, 4 or 8 */
    uint32_t weightedClusterCap;  /* the same for distance-weighted levels: 1..16 (above 8 non-portable) */
    uint32_t useGraphs;           /* 1: each wave's subsampling schedule is captured into one CUDA graph */
    double trialMs;               /* ocpi_batch_autotune: measured time of this choice on its sample */
    uint32_t trials;              /* ocpi_batch_autotune: configurations measured */
    uint32_t lastIssue;           /* set by the library: 1 if the last wave ran as one graph launch */
    uint32_t lanes;               /* 0: waves as above; 1..64: the lane executor (ocpi_batch_build) with this
                                     many lanes, the wave fields unused */
} OcpiBatchTuning;

/* Measures the batched form on an evenly spaced sample of the jobs (at most
 * sampleJobs of them, 0: 256, so that a batch of up to 256 jobs is measured
 * whole: a sample's memory envelope can hide the admission churn of the full
 * batch; their output arrays are written): subsampling
 * waves over a sweep of wave sizes, cluster caps and graph capture, and the
 * lane executor with 4 lanes; returns the fastest in `tuning`.  The choice is kept for the rest of the process per
 * device and batch signature (job count, mean size, share of float64 clouds,
 * of distance-weighted jobs and of 512-grid jobs, each in buckets); with a
 * cachePath it is also read from and appended to that text file, so that a
 * later process starts tuned. */
OCPI_EXPORT int ocpi_batch_autotune(int device, uint64_t memoryBudget, const OcpiJob* jobs, uint32_t count,
                                    uint32_t sampleJobs, const char* cachePath, OcpiBatchTuning* tuning);
/* the batched form with an explicit tuning (waves, or lanes when
   tuning->lanes > 0); tuning->lastIssue is set */
OCPI_EXPORT int ocpi_batch_build_tuned(int device, uint64_t memoryBudget, OcpiBatchTuning* tuning,
                                       const OcpiJob* jobs, uint32_t count, OcpiJobResult* results);

/* ---- allocation-free node subsampling (no counterpart in the reference) --
 *
 * For callers that may not allocate device memory: a plug-in living inside an
 * application whose memory pool owns the whole GPU, or a pipeline that keeps
 * every buffer in a fixed arena.  The session entry points above size and
 * cudaMalloc their buffers; this one subsamples ONE octree node (the
 * per-node step of ocpi_generate_octree) in a fixed scratch array that is
 * part of the library's device image.  It calls no cudaMalloc, cudaFree or
 * allocating library routine.
 *
 * Limits and sharing:
 *   - at most OCPI_NOALLOC_MAX_CANDIDATES candidate points per call; larger
 *     nodes are rejected with -1 and a message in ocpi_last_error();
 *   - the scratch (OCPI_NOALLOC_SCRATCH_BYTES, 12.5 MiB) is held on every GPU
 *     where this library's subsampling module is loaded, until process exit;
 *   - every call shares the scratch and it keeps the last call's contents;
 *     calls that overlap on the GPU (other streams, other host threads) race
 *     and must be ordered by the caller;
 *   - the first call on a device looks up the scratch address on that device
 *     (cudaGetSymbolAddress, with the device current) and may load the
 *     module: make that first call before any stream capture.
 *
 * All pointers named d* / device arrays are device memory of the current
 * device; the call is asynchronous on `stream` (a cudaStream_t, NULL = the
 * legacy default stream).
 *   cloud             device: the point cloud (interleaved records of
 *                     dataStride bytes), readable for 16 bytes past the last
 *                     record
 *   scale, cloudMin   host, 3 doubles: cloud scale and bounding-box minimum
 *   nodeMin, nodeSide host: the node's bounding-box minimum and cube side
 *   level, mortonKey  node level (0 = finest) and its Morton key in the level
 *                     (used by random subsampling)
 *   modeFlags         OCPI_SUB_* bits, as ocpi_configure_subsampling selects
 *   candidateLut      device: cloud index of every candidate point
 *   candidateRecords  device: the candidates' 18-byte octree.bin records,
 *                     readable for 16 bytes past the last record
 *   outLut, outRecords device: room for candidateCount entries / records
 *   outStatus         device, 2 words: [0] points written, [1] error bits
 *                     (1 point below the node box, 4 brick table overflow)
 */
#define OCPI_NOALLOC_MAX_CANDIDATES (131072u)
#define OCPI_NOALLOC_SCRATCH_BYTES (13108480u)
#define OCPI_SUB_INTRA (1u)
#define OCPI_SUB_INTER (2u)
#define OCPI_SUB_RANDOM (8u)
#define OCPI_SUB_WEIGHTING (16u)
OCPI_EXPORT int ocpi_subsample_node_noalloc(const uint8_t* cloud, uint8_t cloudType, uint32_t dataStride,
                                            const double* scale, const double* cloudMin, const double* nodeMin,
                                            double nodeSide, uint32_t level, uint64_t mortonKey,
                                            uint32_t subsamplingGrid, uint32_t modeFlags, uint64_t seed,
                                            const uint32_t* candidateLut, const uint8_t* candidateRecords,
                                            uint32_t candidateCount, uint32_t* outLut, uint8_t* outRecords,
                                            uint32_t* outStatus, void* stream);

#endif /* OCTREE_API_H */
