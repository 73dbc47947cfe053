/*
 * mdmc: Dual Marching Cubes with non-manifold repair on sm_103a (GB300).
 *
 * C ABI of the drop-in boundary for the reference's DMC entry point,
 * PhiliGuertler/ManifoldDMC MarchingCubes/VisualDMC/src/DMC/DualMarchingCubes.h
 * (class DMC::DualMarchingCubes).  Plain pointers and sizes only.  Streams are
 * passed as `void*` holding a cudaStream_t (NULL = the legacy default stream).
 *
 * Citations use the reference's paths relative to
 * MarchingCubes/VisualDMC/src/DMC/.
 *
 * Ownership: every device pointer returned in an mdmc_mesh belongs to the
 * context and stays valid until the next mdmc_run / mdmc_prepare_grid on that
 * context or mdmc_destroy (the reference's algorithm object likewise owns its
 * halfedge mesh until the next run, DualMarchingCubes.h:170-178).
 * A context is used by one host thread at a time.
 */
#ifndef MDMC_H_
#define MDMC_H_

#include <stdint.h>

#if defined(__GNUC__)
#define MDMC_API __attribute__((visibility("default")))
#else
#define MDMC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mdmc_context mdmc_context;

typedef enum mdmc_status {
    MDMC_OK = 0,
    MDMC_ERROR_INVALID_ARGUMENT = 1,
    MDMC_ERROR_CUDA = 2,
    MDMC_ERROR_OUT_OF_MEMORY = 3,
    /* a device-side limit was hit (hash probe limit, partner list overflow,
     * iteration cap); the mesh is still written, see mdmc_last_error */
    MDMC_ERROR_LIMIT = 4,
    MDMC_ERROR_IO = 5,
    MDMC_ERROR_NO_DEVICE = 6
} mdmc_status;

/* SplittingStep, PostProcesses/ManifoldSplitter.h:155-166 */
enum {
    MDMC_STEP_NONE = 0,
    MDMC_STEP_SUBDIVIDE_QUADS = 1,
    MDMC_STEP_COLLAPSE_NON_MANIFOLD_EDGES = 2,
    MDMC_STEP_MERGE_VERTICES = 3,
    MDMC_STEP_UPDATE_HALFEDGE_TWINS = 4,
    MDMC_STEP_MOVE_VERTICES_TO_SURFACE = 5,
    MDMC_STEP_ENABLE_ITERATIVE_REFINEMENT = 6,
    MDMC_STEP_ALL = 100
};

/* Vertex flag bits, Halfedges/Halfedge.h:14-111 */
enum {
    MDMC_VERTEX_NON_MANIFOLD = 1,   /* origin of a 4-face edge's halfedge */
    MDMC_VERTEX_BOUNDARY = 2,       /* origin of a 1-face edge's halfedge */
    MDMC_VERTEX_WEIRD = 4,          /* origin of a 3-face edge's halfedge */
    MDMC_VERTEX_MULTIPLE_FANS = 8   /* non-manifold vertex (more than one face fan) */
};

/* Face attribute bits, DeviceVectors.h:334-450 (QuadrilateralAttribute) */
enum {
    MDMC_FACE_COLOR_MASK = 0x1F,
    MDMC_FACE_NON_MANIFOLD = 0x20,
    MDMC_FACE_PATTERN = 0x40,
    MDMC_FACE_REMOVE = 0x80,
    MDMC_FACE_BOUNDARY = 0x100
};

/* Algorithm flags of DualMarchingCubes (DualMarchingCubes.h:167-185, defaults
 * DualMarchingCubes.cu:110-133) and setSplittingStep (:143-145). */
typedef struct mdmc_options {
    int enable_surface_to_vertex_iteration; /* m_enableSurfaceToVertexIteration, default 1 */
    int simplify_p3x3y_color;                /* m_simplifyP3x3yColor, default 0 */
    int simplify_p3x3y_old;                  /* m_simplifyP3x3yOld, default 0 */
    int simplify_p3333;                      /* m_simplifyP3333, default 0 */
    int split_non_manifold_halfedges;        /* m_splitNonManifoldHalfedges, default 1 */
    int detect_non_manifold_vertices;        /* m_detectNonManifoldVertices, default 1 */
    int splitting_step;                      /* SplittingStep, default MDMC_STEP_ALL */
} mdmc_options;

/* A uniform grid on the device (UniformGrid<float>, UniformGrid.h:44-262):
 * sample (x,y,z) at origin + (x,y,z) * spacing, x fastest in memory.
 * Either dense (samples != NULL, coarse_samples == NULL) or refined and/or
 * padded on demand from a coarse grid (coarse_samples != NULL): the library
 * then evaluates refineGrid's samples where it needs them instead of storing
 * the refined grid.  mdmc_prepare_grid fills this struct. */
typedef struct mdmc_grid {
    const float* samples;
    int32_t dims[3];
    float origin[3];
    float spacing[3];
    const float* coarse_samples;
    int32_t coarse_dims[3];
    int32_t refinement;
    int32_t add_zero_boundary;
} mdmc_grid;

/* The halfedge mesh after post-processing (HalfedgeMesh, Halfedges/HalfedgeMesh.h)
 * as device arrays owned by the context. */
typedef struct mdmc_mesh {
    int64_t num_vertices;   /* vertices, unreferenced ones included */
    int64_t num_faces;
    int64_t num_halfedges;
    float* positions;       /* 3 per vertex */
    float* normals;         /* 3 per vertex */
    int32_t* quads;         /* 4 vertex ids per face, walking next from the first halfedge */
    int32_t* halfedges;     /* 4 per halfedge: origin vertex, face, next, twin (-1 = none) */
    int32_t* face_first_halfedge;
    uint16_t* face_attributes;
    int32_t* vertex_halfedge; /* smallest halfedge leaving the vertex, -1 if none */
    uint8_t* vertex_flags;
} mdmc_mesh;

/* Counters of DualMarchingCubes (DualMarchingCubes.h:87-118) plus timings. */
typedef struct mdmc_stats {
    int64_t num_dmc_vertices;      /* getNumVertices: DMC vertices before repair */
    int64_t num_dmc_quads;         /* getNumQuads */
    int64_t num_active_cells;
    int64_t num_edges;             /* getNumEdges */
    int64_t num_edges3;            /* getNumNonManifoldEdges3 */
    int64_t num_edges4;            /* getNumNonManifoldEdges4 */
    int64_t num_non_manifold_vertices; /* getNumNonManifoldVertices, -1 when detection is off */
    int64_t quads_with_non_manifold_edges[4]; /* getNumQuadsWithNonManifoldEdges(1..4) */
    int64_t split_iterations;
    int64_t anomalies;             /* device-side limit hits, 0 on well-formed input */
    float ms_dmc;                  /* GPU time per stage (CUDA events) */
    float ms_halfedge;
    float ms_repair;
    float ms_detect;
    float ms_total;
    /* per-kernel GPU times of the last run (CUDA events on the run's stream),
     * for the kernels mdmc_set_kernel_timing selects; 0 for the others */
    float ms_refine;               /* grid refinement of the last mdmc_prepare_grid */
    float ms_count;                /* per-row counting pass over the grid */
    float ms_emit;                 /* active-cell compaction pass */
    float ms_vertices;             /* dual vertices of the active cells */
    float ms_quads;                /* quads, halfedges, twins and edge flags (one pass) */
    float ms_table;                /* edge-table rebuilds of the splitter (0: not timed separately) */
    int64_t kernel_launches;       /* kernels launched by the last run and prepare */
} mdmc_stats;

MDMC_API void mdmc_default_options(mdmc_options* options);

/* DualMarchingCubes::DualMarchingCubes, DualMarchingCubes.cu:110-133
 * (+ MarchingCubes::MarchingCubes table upload, :91-98).  options may be NULL. */
MDMC_API mdmc_status mdmc_create(mdmc_context** context, const mdmc_options* options);
/* DualMarchingCubes::~DualMarchingCubes, DualMarchingCubes.cu:135-140 */
MDMC_API void mdmc_destroy(mdmc_context* context);
/* the flag setters of DualMarchingCubes (renderImGui, DualMarchingCubes.cu:150-182;
 * setSplittingStep, DualMarchingCubes.h:143-145) */
MDMC_API mdmc_status mdmc_set_options(mdmc_context* context, const mdmc_options* options);

/* Timing.  Every CUDA event record costs the run's stream about 1.7 us of GPU
 * time on a GB300, so the times are taken only for what the MDMC_TIME_* bits
 * select.  MDMC_TIME_STAGES: the stage times ms_dmc .. ms_total (the
 * reference's Performance result; on by default).  The kernel bits time one
 * kernel each (two records per run; no reference counterpart; off by
 * default).  Fields not timed read 0. */
#define MDMC_TIME_REFINE 1u   /* ms_refine */
#define MDMC_TIME_COUNT 2u    /* ms_count */
#define MDMC_TIME_EMIT 4u     /* ms_emit */
#define MDMC_TIME_QUADS 8u    /* ms_quads */
#define MDMC_TIME_TABLE 16u   /* ms_table */
#define MDMC_TIME_VERTICES 32u /* ms_vertices */
#define MDMC_TIME_STAGES 64u /* ms_dmc, ms_halfedge, ms_repair, ms_detect, ms_total */
#define MDMC_TIME_ALL 127u
MDMC_API mdmc_status mdmc_set_kernel_timing(mdmc_context* context, uint32_t kernels);
MDMC_API mdmc_status mdmc_get_options(const mdmc_context* context, mdmc_options* options);

/* Reads a .bin volume (int32 dims[3], float32 spacing[3], uint16 samples)
 * into host memory as float; origin = -(dims-1)/2 * spacing.  With
 * host_samples == NULL only the header is read.
 * UniformGridHost::readFromFile<unsigned short>, UniformGrid.inl:512-571 */
MDMC_API mdmc_status mdmc_read_bin(const char* path, int32_t dims[3], float spacing[3], float origin[3],
                          float* host_samples);

/* Describes the grid of trilinear refinement by (refinement+1) and/or one
 * layer of replicated boundary samples ("zero boundary") of the input.  The
 * refined grid is evaluated on demand by mdmc_run (bit-identical to the
 * reference's refineGrid output) and not stored.  samples may be a device
 * pointer (samples_on_host = 0), used in place and required to stay valid
 * while the grid is used, or host memory, copied into the context on the
 * stream.  UniformGridHost::readFromFile(file, refinement, addZeroBoundary),
 * UniformGrid.inl:575-608, kernel refineGrid :279-319 */
MDMC_API mdmc_status mdmc_prepare_grid(mdmc_context* context, const float* samples, int samples_on_host,
                              const int32_t dims[3], const float origin[3], const float spacing[3],
                              int32_t refinement, int32_t add_zero_boundary, mdmc_grid* out_grid,
                              void* stream);

/* Writes the dense samples of a grid (refined on demand or not) to a device
 * buffer of dims[0]*dims[1]*dims[2] floats (refineGrid, UniformGrid.inl:279-319). */
MDMC_API mdmc_status mdmc_materialize_grid(mdmc_context* context, const mdmc_grid* grid, float* out, void* stream);

/* DualMarchingCubes::run, DualMarchingCubes.cu:220-289: DMC, halfedge mesh,
 * twin repair, non-manifold split and non-manifold vertex detection as the
 * options say.  mesh and stats may be NULL.  The call returns when the mesh
 * is complete on the stream (it synchronizes on host-side counts). */
MDMC_API mdmc_status mdmc_run(mdmc_context* context, const mdmc_grid* grid, float iso_value, mdmc_mesh* mesh,
                     mdmc_stats* stats, void* stream);

/* The last run's mesh and counters (DualMarchingCubes::getHalfedgeMesh,
 * getVertices and the statistics getters, DualMarchingCubes.h:87-141). */
MDMC_API mdmc_status mdmc_get_mesh(const mdmc_context* context, mdmc_mesh* mesh);
MDMC_API mdmc_status mdmc_get_stats(const mdmc_context* context, mdmc_stats* stats);

/* Copies the last run's mesh to host memory; any pointer may be NULL.  Sizes
 * follow mdmc_mesh.  Synchronous with respect to the stream. */
MDMC_API mdmc_status mdmc_download_mesh(mdmc_context* context, float* positions, float* normals, int32_t* quads,
                               int32_t* halfedges, int32_t* face_first_halfedge,
                               uint16_t* face_attributes, int32_t* vertex_halfedge,
                               uint8_t* vertex_flags, void* stream);

/* Caller-owned host arrays for mdmc_run_to_host, laid out like mdmc_mesh
 * (halfedges: 4 ints per halfedge, 4 halfedges per face), sized for up to
 * capacity_vertices vertices and capacity_faces faces.  Any pointer may be
 * NULL (that array is not copied).  Page-locked memory (cudaMallocHost or
 * cudaHostRegister) lets the copies overlap the run; pageable memory works
 * but copies without overlap. */
typedef struct mdmc_host_mesh {
    int64_t capacity_vertices;
    int64_t capacity_faces;
    float* positions;
    float* normals;
    int32_t* quads;
    int32_t* halfedges;
    int32_t* face_first_halfedge;
    uint16_t* face_attributes;
    int32_t* vertex_halfedge;
    uint8_t* vertex_flags;
} mdmc_host_mesh;

/* DualMarchingCubes::run with the mesh delivered into caller-owned host
 * arrays, the way the reference delivers it into caller-owned buffers
 * (DualMarchingCubes.cu:382-406, there GL buffers): mdmc_run, plus the copies
 * of mdmc_download_mesh, started as soon as each array is final so that they
 * overlap the later stages (halfedges and faces after the quad pass,
 * positions and normals after the vertex pass; arrays a repair stage rewrites
 * are copied again at the end).  The device mesh, mesh and stats are those
 * of mdmc_run.  A mesh larger than the capacities is left on the device and
 * the call returns MDMC_ERROR_LIMIT naming its size.  Synchronous: the host
 * arrays are complete when the call returns. */
MDMC_API mdmc_status mdmc_run_to_host(mdmc_context* context, const mdmc_grid* grid, float iso_value,
                                      const mdmc_host_mesh* out, mdmc_mesh* mesh, mdmc_stats* stats, void* stream);

/* HalfedgeMesh::toVertexAndIndexBuffer (Halfedges/HalfedgeMesh.cu:1102-1146)
 * into device arrays instead of GL buffers (either may be NULL): vertices gets
 * 10 floats per vertex {position[3], normal[3], rgba[4]} with the reference's
 * flag colours (insertVertices :716-760; a vertex without halfedges gets the
 * default Vertex of Mesh.h:15-19: NaN position and normal, magenta), indices
 * gets 6 per face, the triangles (x, y, z) and (z, w, x) of the face's quad
 * (insertHalfedgeFaceIndices :690-714).  Asynchronous on the stream. */
MDMC_API mdmc_status mdmc_render_buffers(mdmc_context* context, float* vertices, uint32_t* indices, void* stream);

/* Writes the last run's mesh as OBJ the way Mesh::writeToFile does
 * (Mesh.cu:446-510): v, vn, then one "f a//a b//b c//c d//d" line per face. */
MDMC_API mdmc_status mdmc_write_obj(mdmc_context* context, const char* path);

/* An indexed triangle mesh in device memory, owned by the context and valid
 * until its next mdmc_run_standard_mc: positions and normals 3 floats per
 * vertex, triangles 3 vertex ids each. */
typedef struct mdmc_triangle_mesh {
    int64_t num_vertices;
    int64_t num_triangles;
    float* positions;
    float* normals;
    int32_t* triangles;
} mdmc_triangle_mesh;

/* Standard Marching Cubes of the older CLI version (standard_mc and
 * map_triangles, MarchingCubes/OriginalDMC/src/DualMarchingCubes.cu:201-328,
 * its hash table VertexHashTable.h:81-113 replaced by an edge bit mask):
 * one vertex per grid edge whose end samples lie on both sides of iso (a
 * sample belongs to the inside when >= iso), at the linear crossing from the
 * edge's low end, with the interpolated central-difference gradients
 * (UniformGrid.h:279-321) divided by their length as its normal; triangles
 * from the reference's t_pattern table.  Vertices are numbered by global edge
 * id 3 * sample + axis, triangles by cell in (z, y, x) order and then table
 * order (the reference numbers both in atomic order).  Refined or padded
 * grids are read through the same on-demand view as mdmc_run.  The
 * context's DMC mesh is left as it was.  Synchronous with respect to the
 * stream; mesh may be NULL. */
MDMC_API mdmc_status mdmc_run_standard_mc(mdmc_context* context, const mdmc_grid* grid, float iso_value,
                                          mdmc_triangle_mesh* mesh, void* stream);

/* Copies the last standard Marching Cubes mesh to host memory; any pointer
 * may be NULL.  Synchronous with respect to the stream. */
MDMC_API mdmc_status mdmc_download_triangle_mesh(mdmc_context* context, float* positions, float* normals,
                                                 int32_t* triangles, void* stream);

/* Face coloring of the older CLI version (FaceColoring::colorFaces,
 * MarchingCubes/OriginalDMC/src/FaceColoring.cu:116-141, kernels :5-116) on
 * the last run's mesh, in place: the color bits (0-4) of the face attributes
 * go from the DMC's 24 grid-edge colors to 0-4.  Classes 5..23 in turn, each
 * face takes the first color of 0..4 that no face across one of its edges
 * holds (the test for 4 skips the fourth neighbour, as at :63); then every
 * face of color 4 takes the first free color of 0..3.  A face whose
 * neighbour has its own class sees that neighbour's color from before the
 * class's pass (the reference reads it live; with a proper grid-edge
 * coloring no two such faces touch).  Asynchronous on the stream. */
MDMC_API mdmc_status mdmc_color_faces(mdmc_context* context, void* stream);

/* quadrilateral_to_triangle (MarchingCubes/OriginalDMC/src/
 * DualMarchingCubes.cu:51-60): quad q = (v0, v1, v2, v3) gives triangles
 * 2q = (v0, v1, v3) and 2q + 1 = (v3, v2, v0).  Device arrays: quads
 * 4 * num_quads ints, triangles 6 * num_quads ints.  Asynchronous. */
MDMC_API mdmc_status mdmc_quads_to_triangles(const int32_t* quads, int64_t num_quads, int32_t* triangles,
                                             void* stream);

/* Mean-ratio element quality (mean_ratio_measure, MarchingCubes/OriginalDMC/
 * src/DualMarchingCubes.cu:93-107; QualityMeasure::mean_ratio,
 * QualityMeasure.h:45-66): per triangle 2 sqrt(3) |(p1-p0) x (p2-p0)| over the
 * sum of its squared edge lengths.  Device arrays; a triangle with a vertex id
 * outside [0, num_vertices) gets NaN and sets *bad_index to 1 (bad_index may
 * be NULL).  Asynchronous on the stream. */
MDMC_API mdmc_status mdmc_mean_ratio(const float* positions, int64_t num_vertices, const int32_t* triangles,
                                     int64_t num_triangles, float* quality, uint32_t* bad_index, void* stream);

/* Adjoint of the last mdmc_run on the context (no counterpart in the
 * reference, which is not differentiable).  Given dL/dpositions (device, 3
 * floats per vertex of the last mesh), writes dL/dsamples for the grid samples
 * the run read: the coarse input for a refined or padded grid, the dense grid
 * otherwise (device, one float per sample; added to the buffer's contents when
 * accumulate != 0, else the buffer is overwritten).  The topology is held
 * fixed; a DMC vertex is origin + (cell + mean of its edge points) * spacing,
 * so the run must have had enable_surface_to_vertex_iteration = 0 (else
 * MDMC_ERROR_INVALID_ARGUMENT).  Vertices appended by the non-manifold split
 * pass their gradient to the DMC vertex they descend from (vertex copies: the
 * copied vertex; subdivision vertices: the face corner they are nearest).
 * The grid's sample buffers must still hold the run's input.  Sums use float
 * atomics, so the last bits can differ from call to call. */
MDMC_API mdmc_status mdmc_backward(mdmc_context* context, const float* dl_dpositions, float* dl_dsamples,
                                   int accumulate, void* stream);

/* Batched form (no counterpart in the reference, whose run takes one grid):
 * n grids of uneven size, each with its iso-value, in one call.  The batch
 * owns one context per grid slot; grid i's mesh and statistics (meshes[i],
 * stats[i], either array may be NULL) stay valid until the next batch run, and
 * mdmc_batch_context(batch, i) gives its context for the other getters.  The
 * pipelines run concurrently on `streams` worker streams; streams = 0 lets the
 * first mdmc_run_batch time 1, 2, 4, 8, 16 and 32 workers on its grids and keep the
 * fastest (mdmc_batch_streams reports the choice); the largest grids start
 * first.  The call waits for the
 * caller's stream (the grids' inputs) first and returns when every mesh is
 * complete.  Grids keep the options given at creation. */
typedef struct mdmc_batch mdmc_batch;
MDMC_API mdmc_status mdmc_batch_create(mdmc_batch** batch, const mdmc_options* options, int streams);
MDMC_API void mdmc_batch_destroy(mdmc_batch* batch);
MDMC_API mdmc_status mdmc_run_batch(mdmc_batch* batch, const mdmc_grid* grids, const float* iso_values, int n,
                                    mdmc_mesh* meshes, mdmc_stats* stats, void* stream);
MDMC_API int mdmc_batch_streams(const mdmc_batch* batch);
MDMC_API mdmc_context* mdmc_batch_context(mdmc_batch* batch, int i);
MDMC_API const char* mdmc_batch_last_error(const mdmc_batch* batch);

/* Human-readable description of the context's last error ("" if none). */
MDMC_API const char* mdmc_last_error(const mdmc_context* context);

/* Volume generators (UniformGridHost::generateVolume / generateEdgeCase,
 * UniformGrid.inl:20-269, :463-509).  surface_case follows SurfaceCase
 * (UniformGrid.h:26-37): 0 sphere, 1 torus, 2 two-holed torus, 3 four-holed
 * torus, 4 genus two, 5 iWP, 6 pwHybrid, 7 neovius, 8 Goursat, 9 Steiner's
 * Roman surface.  Samples the surface on [-1, 1]^3 into a device buffer of
 * dims[0]*dims[1]*dims[2] floats and reports the grid's origin and spacing.
 * The edge cases (which = 0, 1: NonManifoldVertex0/1) are 4x4x3 grids of
 * 850/950.  Asynchronous on the stream. */
MDMC_API mdmc_status mdmc_generate_volume(int32_t surface_case, const int32_t dims[3], float* samples,
                                          float origin[3], float spacing[3], void* stream);
MDMC_API mdmc_status mdmc_generate_edge_case(int32_t which, float* samples, int32_t dims[3], float origin[3],
                                             float spacing[3], void* stream);

/* Writes a .bin volume (int32 dims[3], float32 spacing[3], then the samples
 * cast to uint16, x fastest), the format mdmc_read_bin reads
 * (UniformGridHost::writeSelectionToFile<unsigned short> over the whole grid,
 * UniformGrid.inl:632-695).  host_samples is host memory. */
MDMC_API mdmc_status mdmc_write_bin(const char* path, const int32_t dims[3], const float spacing[3],
                                    const float* host_samples);

/* Build-time tables, for tests: the packed contour word of every Marching
 * Cubes case and whether the case takes the asymptotic-decider path.  No
 * reference counterpart (the reference keeps them in s_polygonPatterns and
 * s_triangleAmbiguities, DualMarchingCubes.cpp:301,564). */
MDMC_API void mdmc_case_tables(uint64_t contour_words[256], uint8_t ambiguous[256]);

/* Nearest points for the differentiable form's Chamfer loss (no
 * counterpart in the reference).  mdmc_point_index_create copies `count`
 * points (device memory, 3 floats each), sorts them along a Morton curve on
 * the host and keeps them in device memory the index owns until
 * mdmc_point_index_destroy.  Synchronous. */
typedef struct mdmc_point_index mdmc_point_index;
MDMC_API mdmc_status mdmc_point_index_create(mdmc_point_index** index, const float* points, int64_t count,
                                             void* stream);
MDMC_API void mdmc_point_index_destroy(mdmc_point_index* index);
/* For each of `count` query points (device, 3 floats each): the index of the
 * nearest indexed point (its position in the array given to create) and,
 * when dist2 is not NULL, the squared distance (dx*dx + dy*dy) + dz*dz in
 * float.  Exact: equal distances go to the smaller index.  The points are
 * kept in tiles along a Morton curve; a tile whose bounding box is farther
 * from a query than the query's best distance so far (strictly) is not
 * compared, which never skips the nearest point or a tie.
 * scratch: device memory of 2 * count + 2056 uint64 the call overwrites.
 * Asynchronous on the stream. */
MDMC_API mdmc_status mdmc_point_index_nearest(const mdmc_point_index* index, const float* queries, int64_t count,
                                              int32_t* nearest, float* dist2, uint64_t* scratch, void* stream);
/* The number of indexed points. */
MDMC_API int64_t mdmc_point_index_count(const mdmc_point_index* index);

/* The count pass of mdmc_run without a context and without allocating:
 * writes {active cells, DMC quads} of the grid at iso_value to totals, two
 * int64 in DEVICE memory, asynchronously on the stream (equal to
 * mdmc_stats.num_active_cells and num_dmc_quads of an mdmc_run).  This entry
 * point has no counterpart in the reference.  It is for callers that cannot
 * allocate device memory: code that sizes its buffers inside a stream or frame
 * loop with a fixed device-memory pool, or that must not stall the device
 * (cudaMalloc/cudaFree synchronize it, and mdmc_run grows its buffers with
 * them).  Its scratch is a fixed device array shared by every call on a
 * device: at most 2^18 x-rows of cells ((dims[1]-1)*(dims[2]-1)) and, for a
 * refined grid, 2^24 coarse cells; larger grids return MDMC_ERROR_LIMIT before
 * any work.  Calls that overlap on the GPU race on the scratch: serialize
 * them.  The first call on a device (with that device current) looks up the
 * scratch there, which loads this code onto the device; make it before any
 * stream capture.  After a cudaDeviceReset the next call on that device finds
 * a new context and looks the scratch up again (a set-up call once more).
 * message (may be NULL) receives an error description of at
 * most message_len bytes. */
MDMC_API mdmc_status mdmc_count_cells_noalloc(const mdmc_grid* grid, float iso_value, int64_t* totals, void* stream,
                                              char* message, int message_len);

#ifdef __cplusplus
}
#endif

#endif /* MDMC_H_ */
