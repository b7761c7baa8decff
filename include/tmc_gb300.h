/* tmc_gb300: uniform-grid isosurface extraction on one GB300 (sm_103a).
 *
 * C ABI over hand-written CUDA kernels.  Plain C types only; every entry point returns a
 * tmc_status and never exits the process.  The entry points replace these reference calls:
 *
 *   tmc_dmc_extract        dmc::DualMarchingCubes::dualMC          cpp_dmc/DualMarchingCubes.h:163-165
 *                          p_mc::DualMarchingCubes::dualMC          dmc/DualMarchingCubes.h:74-77
 *   tmc_tmc_sharedvertex   p_mc::MarchingCubes::mc_sharedvertex     cuda_tmc/MarchingCubes.h:60
 *                          tmc::MarchingCubes::t_mc (via operator()) mc/MarchingCubes.h:301, mc/MarchingCubes.cpp:151
 *   tmc_tmc_halfedge       p_mc::MarchingCubes::mc_halfedge         cuda_tmc/MarchingCubes.h:71
 *   tmc_batch_extract      (no single reference call: many dualMC / mc_sharedvertex calls in one launch)
 *   tmc_server_*           (no reference counterpart: request loop around the calls above)
 *   tmc_dmc_count_static   (no reference counterpart: DMC mesh sizes without allocating)
 *   tmc_dmc_color_valence  colorFaces + vertexValence                cpp_dmc/DualMarchingCubes.cpp:714-871
 *   tmc_ctx_*_tuning, tmc_ctx_autotune  (no reference counterpart: launch shapes and their tuner)
 *   tmc_field_load         dmc::UniformGrid::init(file)              cpp_dmc/UniformGrid.cpp:3-45
 *                          readFromFile<T> / readDataFromFile<T>     cpp_dmc/Volumes.h:47, dmc/UniformGrid.h:431
 *                          p_mc::MarchingCubes::readDataFromFile    cuda_tmc/MarchingCubes.cu:3363
 *   tmc_field_generate     p_mc::UniformGrid::generateVolume         dmc/UniformGrid.cu:177-217
 *   tmc_field_generate_ex, tmc_*_extract_generated  (no reference counterpart: parameterised fields,
 *                          generation fused into the extraction)
 *   tmc_mesh_write_obj/off the OBJ / OFF writers                     cpp_dmc/main.cpp:33-87, mc/MarchingCubes.cpp:98-141
 *   tmc_mesh_quality       p_mc::EstimateElementQuality::q           dmc/EstimateElementQuality.cu:39-56
 *   tmc_mesh_valence       p_mc::VertexValence::vertexValence        dmc/VertexValence.cu:79-170
 *   tmc_mesh_check         tmc::MarchingCubes::connectivity (counts) mc/MarchingCubes.cpp:1769-2226
 *
 * Threading: a context is thread-compatible, not thread-safe; use one context per host thread.
 * All work of a context runs on its own CUDA stream.
 */
#ifndef TMC_GB300_H
#define TMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tmc_status {
  TMC_OK = 0,
  TMC_ERR_INVALID_ARG = 1, /* null pointer, bad size, unknown flag */
  TMC_ERR_OOM = 2,         /* device or host allocation failed */
  TMC_ERR_CAPACITY = 3,    /* a fixed-capacity buffer overflowed (batched/served paths) */
  TMC_ERR_CUDA = 4,        /* a CUDA runtime call failed; see tmc_last_error */
  TMC_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  TMC_ERR_NUMERIC = 6,     /* the field holds NaN or Inf */
  TMC_ERR_INTERNAL = 7
} tmc_status;

typedef struct tmc_ctx tmc_ctx;

typedef struct tmc_ctx_opts {
  size_t reserve_bytes; /* device memory the context keeps pooled between calls (0 = default) */
  int32_t check_numeric; /* 1: scan the field for NaN/Inf and fail with TMC_ERR_NUMERIC */
  /* stream priority of the context's work: 0 = default; a negative value lets its kernels take
   * SMs ahead of other streams' work (clamped to cudaDeviceGetStreamPriorityRange) */
  int32_t priority;
} tmc_ctx_opts;

/* A uniform grid: point (i,j,k) sits at origin + (i,j,k)*spacing; data[(k*ny + j)*nx + i]. */
typedef struct tmc_volume {
  int32_t nx, ny, nz;   /* grid points per axis, each >= 2 */
  double origin[3];
  double spacing[3];
  const float* data;    /* float32 scalar field, x fastest */
  int32_t on_device;    /* 1: `data` is device memory on the context's device; 0: host memory */
  int32_t reserved;
} tmc_volume;

/* flags */
enum {
  /* DMC mesh simplification, as cpp_dmc's sFlag (DualMarchingCubes.cpp:60-72): P3X3Y colour pass,
   * P3X3Y isolated pass and P3333.  The three can also be chosen one by one. */
  TMC_DMC_SIMPLIFY = 1u << 0,
  TMC_DMC_P3X3Y_COLOR = 1u << 1,
  TMC_DMC_P3X3Y_ISOLATED = 1u << 2,
  TMC_DMC_P3333 = 1u << 3,
  TMC_OUT_TRIANGLES = 1u << 4,  /* DMC: also split quads into triangles (collectTriangles) */
  TMC_OUT_HALFEDGES = 1u << 5,  /* halfedges {origin, face, next, twin} + vertex/face handles */
  TMC_OUT_HOST = 1u << 6,       /* results in host memory (owned by the mesh) instead of device */
  TMC_OUT_POS_F64 = 1u << 7,    /* also emit float64 positions, bit-equal to the CPU reference */
  TMC_OUT_LOCAL = 1u << 8,      /* DMC without simplification: per-vertex generating cell + local (u,v,w) */
  TMC_GRAD_FLIP = 1u << 9,      /* DMC normals from the negated gradient (UniformGrid::flip_gradient) */
  TMC_TMC_KEY32 = 1u << 10      /* TMC: reproduce the reference's 32-bit edge keys (int overflow included) */
};

typedef struct tmc_mesh {
  int64_t nr_v, nr_q, nr_t, nr_he;
  int32_t on_device; /* 1: arrays are device pointers (valid until tmc_mesh_free) */
  int32_t reserved;
  float* v;          /* 3*nr_v positions */
  float* n;          /* 3*nr_v unit normals */
  double* v64;       /* 3*nr_v float64 positions (TMC_OUT_POS_F64), else NULL */
  int32_t* quads;    /* 4*nr_q (DMC) */
  int32_t* tris;     /* 3*nr_t */
  int32_t* he;       /* 4*nr_he: origin, face, next, twin (-1 = boundary) */
  int32_t* he_v;     /* nr_v: one outgoing halfedge per vertex */
  int32_t* he_f;     /* per face: its first halfedge */
  int64_t* vcell;    /* nr_v generating cell (TMC_OUT_LOCAL) */
  float* vuvw;       /* 3*nr_v local coordinates in the generating cell (TMC_OUT_LOCAL) */
  int64_t stats[8];  /* [0] active cells [1] ambiguous cells [2,3] representative fallbacks
                        (7x7 then 26x26 failed) [4] non-manifold edges [5] singular faces [6] cells
                        [7] values the DMC vertex kernel recomputed in float64 (samples, normals) */
  void* priv;
} tmc_mesh;

/* context ---------------------------------------------------------------------------------- */
tmc_status tmc_ctx_create(int device, const tmc_ctx_opts* opts, tmc_ctx** out);
tmc_status tmc_ctx_destroy(tmc_ctx* ctx);
const char* tmc_last_error(const tmc_ctx* ctx);
void* tmc_ctx_stream(tmc_ctx* ctx); /* the context's cudaStream_t */
tmc_status tmc_ctx_synchronize(tmc_ctx* ctx);
/* number of library kernels launched by this context since creation */
int64_t tmc_ctx_launch_count(const tmc_ctx* ctx);
/* Per-stage device timing with CUDA events on the context stream (the counterpart of the
 * reference's CTimer stage report, dmc/CTimer.h:123-190).  Enabling resets the totals. */
tmc_status tmc_ctx_set_profiling(tmc_ctx* ctx, int on);
/* Copies up to `max` stages: names (32 chars each), accumulated milliseconds and event counts.
 * Returns the number of stages, or -1. */
int32_t tmc_ctx_profile_read(tmc_ctx* ctx, int32_t max, char* names, double* ms, int64_t* counts);

/* Launch shapes (no reference counterpart: the reference's kernels use fixed launch sizes).  Every
 * setting gives identical meshes; the settings trade the latency of small calls against the
 * throughput of large ones.  Defaults follow the device's SM count; tmc_ctx_autotune measures. */
enum {
  TMC_TUNE_GROUP_LANES = 1,          /* lanes the DMC projection pass may fill with a group of lanes
                                        per vertex (small meshes); 0 = one thread per vertex */
  TMC_TUNE_WARP_LIST_MAX = 2,        /* DMC float64-fallback lists up to this length run one warp
                                        per vertex (0 = one thread per vertex, retries by warp) */
  TMC_TUNE_VERTEX_BLOCKS_PER_SM = 3, /* grid cap of the per-vertex DMC passes, 1..64 */
  TMC_TUNE_EMIT_BLOCKS_PER_SM = 4,   /* grid cap of the TMC emission kernel, 1..64 */
  /* the slab pipeline of a host field (copy of slab q+1 beside the classification of slab q):
   * slab depth in MiB (4..1024) and the most slabs per field (2..64) */
  TMC_TUNE_SLAB_MIB = 5,
  TMC_TUNE_MAX_SLABS = 6,
  TMC_TUNE_QUAD_BLOCKS_PER_SM = 7    /* grid of the DMC quad pass over the listed cells, 1..64 */
};
tmc_status tmc_ctx_set_tuning(tmc_ctx* ctx, int32_t key, int64_t value);
tmc_status tmc_ctx_get_tuning(const tmc_ctx* ctx, int32_t key, int64_t* value);

/* extraction -------------------------------------------------------------------------------- */
/* Dual Marching Cubes: quad mesh (+ triangles, + halfedges).  Vertices in generating-cell order,
 * quads in dual-edge key order, as the reference CPU path emits them. */
tmc_status tmc_dmc_extract(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out);
/* Topologically correct Marching Cubes, shared-vertex triangle mesh. */
tmc_status tmc_tmc_sharedvertex(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out);
/* Topologically correct Marching Cubes with the triangle halfedge structure. */
tmc_status tmc_tmc_halfedge(tmc_ctx* ctx, const tmc_volume* vol, double iso, uint32_t flags, tmc_mesh* out);
tmc_status tmc_mesh_free(tmc_ctx* ctx, tmc_mesh* mesh);

/* Sizes of a DMC extraction without allocating (no counterpart in the reference).
 * counts[0] vertices, [1] quads: tmc_dmc_extract's nr_v and nr_q without simplification flags;
 * counts[2] active cells, [3] ambiguous cells: its stats[0] and stats[1].
 * For callers that must not allocate device memory at call time, e.g. a server sizing a mesh
 * before admitting the request against a fixed memory budget.  The field must be device memory.
 * Scratch is one static 512 KiB device array per device: grids above 134,217,728 cells (513^3
 * points) fail with TMC_ERR_CAPACITY; calls overlapping in time on one device race on the array
 * and must be serialised; every call looks up the array's address (cudaGetSymbolAddress), and
 * the first call on a device may load the library's device code there, so it should precede any
 * stream capture on that device.  Volumes are checked as tmc_dmc_extract checks them. */
tmc_status tmc_dmc_count_static(tmc_ctx* ctx, const tmc_volume* vol, double iso, int64_t counts[4]);

/* The face colouring and vertex valence stage of the DMC simplification on its own: the
 * reference's colorFaces + vertexValence (cpp_dmc/DualMarchingCubes.cpp:714-871; GPU counterparts
 * p_mc::FaceColoring::colorFaces, dmc/FaceColoring.cu:121-145, and vertexValence,
 * dmc/MeshSimplification.cu:45-59).  quads: 4*nr_q vertex ids of a quad mesh; colors: nr_q
 * inherited colours (3*parity + axis of the dual grid edge, 0..23) on entry, the reduced colours
 * (0..4) on return; valence: nr_v counts out.  All three are device arrays; the call returns when
 * they are written. */
tmc_status tmc_dmc_color_valence(tmc_ctx* ctx, int64_t nr_v, int64_t nr_q, const int32_t* quads, uint8_t* colors,
                                 int32_t* valence);

/* volume files and mesh files --------------------------------------------------------------- */
/* The reference's volume file layouts (origin 0; the data x fastest):
 *   TMC_FILE_DMC      int32 nx,ny,nz; float64 dx,dy,dz; float32 data   cpp_dmc/UniformGrid.cpp:3-45
 *   TMC_FILE_INT_F32  int32 nx,ny,nz; float32 dx,dy,dz; float32 data   cpp_dmc/Volumes.h:47-105,
 *                                                                      dmc/UniformGrid.h:431-468
 *   TMC_FILE_INT_U16  int32 nx,ny,nz; float32 dx,dy,dz; uint16 data    (their ushort instances)
 *   TMC_FILE_U16      uint16 nx,ny,nz; float32 dx,dy,dz; uint16 data   mc/MarchingCubes.cpp:22-66,
 *                                                                      cuda_tmc/MarchingCubes.cu:3363-3407 */
enum { TMC_FILE_DMC = 0, TMC_FILE_INT_F32 = 1, TMC_FILE_INT_U16 = 2, TMC_FILE_U16 = 3 };
/* A field loaded into device memory; `vol` describes it (on_device = 1) until tmc_field_free. */
typedef struct tmc_field {
  tmc_volume vol;
  void* priv;
} tmc_field;
/* Header of a volume file: dimensions, spacing (float64) and the offset of the first data byte.
 * Checks that the file holds all the data it announces.  Needs no context and no GPU. */
tmc_status tmc_volume_file_info(const char* path, int32_t format, int32_t dims[3], double spacing[3],
                                int64_t* data_offset);
/* Reads a volume file into device memory as float32 (uint16 data is copied as it is and widened on
 * the GPU).  Replaces the reference's readers, which exit the process on a bad file. */
tmc_status tmc_field_load(tmc_ctx* ctx, const char* path, int32_t format, tmc_field* out);
tmc_status tmc_field_free(tmc_ctx* ctx, tmc_field* field);
/* The reference's predefined implicit surfaces (p_mc::UniformGrid::generateVolume,
 * dmc/UniformGrid.cu:21-217) sampled on the GPU on [-1, 1]^3 (spacing 2 / (n - 1) in float32, as the
 * reference), into device memory; free with tmc_field_free.  Isovalue 0 for every surface. */
enum {
  TMC_SURF_SPHERE = 0, TMC_SURF_TORUS = 1, TMC_SURF_TWO_HOLED_TORUS = 2, TMC_SURF_FOUR_HOLED_TORUS = 3,
  TMC_SURF_GENUS_TWO = 4, TMC_SURF_IWP = 5, TMC_SURF_PW_HYBRID = 6, TMC_SURF_NEOVIUS = 7, TMC_SURF_GOURSAT = 8,
  TMC_SURF_STEINER_ROMAN = 9
};
tmc_status tmc_field_generate(tmc_ctx* ctx, int32_t surface, int32_t nx, int32_t ny, int32_t nz, tmc_field* out);
/* Generated fields with parameters (no counterpart in the reference's API: the two field families of
 * the batched workloads, evaluated in float32 on the same grid):
 *   TMC_SURF_PERIODIC  sin(kx)cos(ky) + sin(ky)cos(kz) + sin(kz)cos(kx), k = params[0]
 *   TMC_SURF_BLOBS     sum over `count` (1..16) blobs of exp(-|p - c|^2 / (2 sigma^2)), blob b:
 *                      params[4b .. 4b+2] = centre, params[4b+3] = sigma
 * and the ten surfaces above (params unused). */
enum { TMC_SURF_PERIODIC = 10, TMC_SURF_BLOBS = 11 };
typedef struct tmc_generator {
  int32_t surface;     /* TMC_SURF_* */
  int32_t nx, ny, nz;  /* points on [-1, 1]^3, spacing 2 / (n - 1) in float32 */
  int32_t count;       /* TMC_SURF_BLOBS: number of blobs */
  int32_t reserved;
  double params[64];
} tmc_generator;
/* The generator's field written to device memory (the stored path); free with tmc_field_free. */
tmc_status tmc_field_generate_ex(tmc_ctx* ctx, const tmc_generator* gen, tmc_field* out);
/* Extraction with the field generation fused into the classification: the classification kernels
 * evaluate the field instead of reading it (each point once) and keep the values for the passes
 * that follow, which touch only the crossed cells' neighbourhoods; no generation pass and no field
 * read.  The meshes equal those of tmc_field_generate_ex followed by tmc_dmc_extract /
 * tmc_tmc_sharedvertex / tmc_tmc_halfedge (halfedge != 0) on the same field, bit for bit. */
tmc_status tmc_dmc_extract_generated(tmc_ctx* ctx, const tmc_generator* gen, double iso, uint32_t flags,
                                     tmc_mesh* out);
tmc_status tmc_tmc_extract_generated(tmc_ctx* ctx, const tmc_generator* gen, double iso, uint32_t flags,
                                     int32_t halfedge, tmc_mesh* out);
/* OBJ output in the reference's layouts: TMC_OBJ_DMC_TRIS / TMC_OBJ_DMC_QUADS as cpp_dmc/main.cpp:33-87
 * (the triangle or the quad file), TMC_OBJ_TMC as mc/MarchingCubes.cpp:98-118 (including its use of
 * the second vertex's index as the third normal index).  OFF output as mc/MarchingCubes.cpp:123-141
 * (a mesh with quads and no triangles writes 4-vertex faces).  Positions are written from the
 * float64 array when the mesh has one.  ctx may be NULL for a mesh in host memory. */
enum { TMC_OBJ_DMC_TRIS = 0, TMC_OBJ_DMC_QUADS = 1, TMC_OBJ_TMC = 2 };
tmc_status tmc_mesh_write_obj(tmc_ctx* ctx, const tmc_mesh* mesh, const char* path, int32_t style);
tmc_status tmc_mesh_write_off(tmc_ctx* ctx, const tmc_mesh* mesh, const char* path);

/* mesh validation metrics (the reference's validation kernels, not part of its extraction path) -- */
enum { TMC_FACES_QUADS = 0, TMC_FACES_TRIS = 1 };
/* Element quality as p_mc::EstimateElementQuality (dmc/EstimateElementQuality.cu:1-56,
 * dmc/ElementQuality.h:69-93): per quad the smallest 2|e1 x e2| / (|e1|^2 + |e2|^2) over its corners,
 * per triangle the mean ratio 2 sqrt(3)|e1 x e2| / (l0 + l1 + l2) (0 with a zero-length edge), float32.
 * quality (host, one per face) and summary (host: min, max, mean) may each be NULL.  The mesh may be
 * in host or device memory. */
tmc_status tmc_mesh_quality(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, float* quality, double summary[3]);
/* Valence distribution as p_mc::VertexValence::vertexValence (dmc/VertexValence.cu:79-170):
 * hist[k] = number of vertices with k distinct incident edges (k = 99 also counts higher valences);
 * *len = the last non-empty bin + 1, as the reference trims its vector. */
tmc_status tmc_mesh_valence(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, uint32_t hist[100], int32_t* len);
/* Mesh check, the counts of tmc::MarchingCubes::connectivity (mc/MarchingCubes.cpp:1769-2226), which
 * repairs orientation in a sequential walk; here a parallel validator that changes nothing:
 * report[0] connected components (faces joined across shared edges), [1] orientation defects (edges
 * whose two faces run them in the same direction; 0 on a consistently oriented mesh, where the
 * reference flips nothing), [2] boundary edges, [3] halfedges on non-manifold edges,
 * [4] degenerate faces (a repeated vertex), [5] boundary vertices. */
tmc_status tmc_mesh_check(tmc_ctx* ctx, const tmc_mesh* mesh, int32_t faces, int64_t report[6]);

/* batched extraction ------------------------------------------------------------------------ */
enum { TMC_ALGO_DMC = 0, TMC_ALGO_TMC = 1 };
typedef struct tmc_request {
  tmc_volume vol;
  double iso;
  uint32_t algo;  /* TMC_ALGO_DMC or TMC_ALGO_TMC */
  uint32_t flags;
} tmc_request;
/* Extract n independent requests in one batched pipeline (device-resident fields). */
tmc_status tmc_batch_extract(tmc_ctx* ctx, int32_t n, const tmc_request* reqs, tmc_mesh* outs);
/* Autotuner (no reference counterpart): times `rounds` batched extractions of the given requests
 * for each candidate launch shape (coordinate descent over the TMC_TUNE_* keys) and keeps the
 * fastest in the context; *best_ms (optional) receives the time of one batch with the result.  With
 * one request the single-volume entry point is timed instead, and a host field there also tunes the
 * slab pipeline (TMC_TUNE_SLAB_MIB, TMC_TUNE_MAX_SLABS). */
tmc_status tmc_ctx_autotune(tmc_ctx* ctx, int32_t n, const tmc_request* reqs, int32_t rounds, double* best_ms);

/* request server (no reference counterpart) ------------------------------------------------------
 * Continuous batching: clients submit requests from any thread; worker threads (one stream each)
 * take the oldest pending requests whenever they are free, as many as the HBM budget and the batch
 * limit admit, and run them as one batched extraction, so several batches are in flight at once.
 * A request's field must stay valid until its ticket completes.  Each mesh equals the mesh of the
 * same request extracted alone. */
typedef struct tmc_server tmc_server;
typedef struct tmc_server_opts {
  size_t hbm_budget;  /* device bytes admitted requests may use at once, by estimate (0 = 120 GiB) */
  int32_t workers;    /* batches in flight, one CUDA stream each (0 = 2) */
  int32_t max_batch;  /* requests per batch (0 = 64) */
  int32_t reserved;
  int64_t max_batch_cells; /* cells per batch (0 = 2^25); a larger request runs alone.  The requests of
                              a batch complete together: the cap bounds how long a small request
                              waits for the large ones batched with it */
} tmc_server_opts;
tmc_status tmc_server_create(int device, const tmc_server_opts* opts, tmc_server** out);
tmc_status tmc_server_destroy(tmc_server* server);
tmc_status tmc_server_submit(tmc_server* server, const tmc_request* req, int64_t* ticket);
/* *done = 1 once the ticket's mesh (or error) is ready */
tmc_status tmc_server_poll(tmc_server* server, int64_t ticket, int32_t* done);
/* Blocks until the ticket completes (timeout_s < 0: no limit; TMC_ERR_TIMEOUT when it runs out) and
 * hands over its mesh (mesh.reserved records the worker that owns it). */
tmc_status tmc_server_wait(tmc_server* server, int64_t ticket, double timeout_s, tmc_mesh* out);
tmc_status tmc_server_release(tmc_server* server, tmc_mesh* mesh);
const char* tmc_server_last_error(const tmc_server* server);
/* [0] submitted [1] completed [2] batches [3] requests in batches [4] peak admitted bytes
 * [5] largest batch [6] pending now [7] admitted bytes now */
tmc_status tmc_server_stats(tmc_server* server, int64_t out[8]);

#ifdef __cplusplus
}
#endif
#endif /* TMC_GB300_H */
