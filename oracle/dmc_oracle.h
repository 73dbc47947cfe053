/*
 * CPU oracle for the Dual Marching Cubes + manifold repair path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates the reference's algorithm
 * (PhiliGuertler/ManifoldDMC, MarchingCubes/VisualDMC/src/DMC/) on the CPU so
 * that the CUDA path can be checked against it.  Only tests/, the smoke test
 * and bench.py's CPU-baseline leg may load it.  The product library never
 * links or calls it.
 *
 * Parity pin: the oracle is checked against the reference's 28 golden meshes
 * (Data-and-Results/Base-Results) in tests/test_oracle_golden.py.
 *
 * Ordering conventions (the reference's are atomic-order nondeterministic; the
 * oracle and the CUDA path share these deterministic ones):
 *   - vertices: by cell linear index, then contour index inside the cell;
 *   - quads: by edge key 3*sample_index + axis, ascending;
 *   - halfedge 4q+i belongs to quad q; halfedge ids inside an edge bucket are
 *     sorted ascending before twins are formed;
 *   - splitter working copies: non-manifold faces in ascending face order,
 *     new elements per face in the reference's per-thread creation order.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mdmc_oracle_options {
    int surface_iteration;     /* m_enableSurfaceToVertexIteration (default 1) */
    int simplify_3x3y_color;   /* m_simplifyP3x3yColor (default 0) */
    int simplify_3x3y_old;     /* m_simplifyP3x3yOld (default 0) */
    int simplify_3333;         /* m_simplifyP3333 (default 0) */
    int split_non_manifold;    /* m_splitNonManifoldHalfedges (default 1) */
    int detect_non_manifold_vertices; /* m_detectNonManifoldVertices (default 1) */
    int splitting_step;        /* SplittingStep, 100 = All (default) */
} mdmc_oracle_options;

/* counts[] layout of mdmc_oracle_counts */
enum {
    MDMC_ORC_NUM_VERTICES = 0,
    MDMC_ORC_NUM_FACES = 1,
    MDMC_ORC_NUM_HALFEDGES = 2,
    MDMC_ORC_NUM_DMC_VERTICES = 3,   /* before post-processing */
    MDMC_ORC_NUM_DMC_QUADS = 4,
    MDMC_ORC_NUM_COUNTS = 5
};

/* stats[] layout of mdmc_oracle_stats (mirrors the reference's getters) */
enum {
    MDMC_ORC_STAT_EDGES = 0,          /* getNumEdges */
    MDMC_ORC_STAT_EDGES3 = 1,         /* getNumNonManifoldEdges3 */
    MDMC_ORC_STAT_EDGES4 = 2,         /* getNumNonManifoldEdges4 */
    MDMC_ORC_STAT_NM_VERTICES = 3,    /* getNumNonManifoldVertices (-1 if detection off) */
    MDMC_ORC_STAT_QUADS_NM1 = 4,      /* getNumQuadsWithNonManifoldEdges(1..4) */
    MDMC_ORC_STAT_QUADS_NM2 = 5,
    MDMC_ORC_STAT_QUADS_NM3 = 6,
    MDMC_ORC_STAT_QUADS_NM4 = 7,
    MDMC_ORC_STAT_SPLIT_ITERATIONS = 8,
    MDMC_ORC_STAT_ANOMALIES = 9,      /* bitmask: 2 slot conflict, 4 bucket overflow, 8 partner overflow,
                                         16 fan-walk cap, 32 twin outside copy, 64 iteration cap,
                                         128 wall outside grid, 512 mapping swap */
    MDMC_ORC_NUM_STATS = 10
};

void mdmc_oracle_default_options(mdmc_oracle_options* o);

/* Reads a reference .bin volume (int32 dims[3], float32 spacing[3], uint16
 * samples, x fastest); origin = -(dims-1)/2 * spacing.  With out == NULL only
 * the header is returned.  Returns 0 on success.  D/UniformGrid.inl:512-571 */
int mdmc_oracle_read_bin(const char* path, int dims[3], float spacing[3], float origin[3], float* out);

/* Trilinear refinement and/or replicate padding, D/UniformGrid.inl:279-319 and
 * :575-608.  out must hold the refined dims' product; out_dims, out_origin and
 * out_spacing receive the refined grid's geometry. */
void mdmc_oracle_refine(const float* in, const int dims[3], const float origin[3],
                        const float spacing[3], int refinement, int pad,
                        float* out, int out_dims[3], float out_origin[3], float out_spacing[3]);

void* mdmc_oracle_run(const float* grid, const int dims[3], const float origin[3],
                      const float spacing[3], float iso, const mdmc_oracle_options* opt);
/* mdmc_oracle_refine followed by mdmc_oracle_run, the refined grid kept in
 * the arithmetic type (float, or double in the FP64 build). */
void* mdmc_oracle_run_refined(const float* coarse, const int dims[3], const float origin[3],
                              const float spacing[3], int refinement, int pad, float iso,
                              const mdmc_oracle_options* opt);
void mdmc_oracle_counts(const void* result, int64_t counts[MDMC_ORC_NUM_COUNTS]);
void mdmc_oracle_stats(const void* result, int64_t stats[MDMC_ORC_NUM_STATS]);
/* Any pointer may be NULL.  halfedges: 4 ints per halfedge (origin, face, next, twin). */
void mdmc_oracle_get(const void* result, float* positions, float* normals, int* halfedges,
                     int* face_first, uint16_t* face_attr, uint8_t* vertex_flags, int* vertex_he);
/* DMC stage only (before post-processing): vertices and quads (4 ids). */
void mdmc_oracle_get_dmc(const void* result, float* positions, float* normals, int* quads,
                         uint16_t* quad_attr);
void mdmc_oracle_free(void* result);

/* Standard Marching Cubes of the older CLI version (OriginalDMC standard_mc,
 * O/DualMarchingCubes.cu:201-328): vertices by global edge id 3 * sample +
 * axis, triangles by cell then table order.  counts = {vertices, triangles}. */
void* mdmc_oracle_standard_mc(const float* grid, const int dims[3], const float origin[3], const float spacing[3],
                              float iso, int64_t counts[2]);
void mdmc_oracle_get_standard_mc(const void* mesh, float* positions, float* normals, int* triangles);
void mdmc_oracle_free_standard_mc(void* mesh);

/* Face coloring 24 -> 5 colors in place (O/FaceColoring.cu:5-141);
 * halfedges 4 ints each {origin, face, next, twin}. */
void mdmc_oracle_color_faces(const int32_t* halfedges, int64_t num_halfedges, const int32_t* face_first,
                             uint16_t* face_attr, int64_t num_faces);
/* quadrilateral_to_triangle (O/DualMarchingCubes.cu:51-60) */
void mdmc_oracle_quads_to_triangles(const int32_t* quads, int64_t num_quads, int32_t* tris);
/* mean-ratio quality per triangle (O/QualityMeasure.h:45-66) */
void mdmc_oracle_mean_ratio(const float* pos, const int32_t* tris, int64_t num_triangles, float* q);

/* Differentiable path (no reference counterpart; surface iteration off).
 * Topology of a result: per DMC vertex its cell (x, y, z) and the 12-bit mask
 * of its contour's cell edges; per final vertex the DMC vertex it descends
 * from (itself for DMC vertices, the corner vertex for split vertices, -1 if
 * none).  Any pointer may be NULL. */
void mdmc_oracle_get_topology(const void* result, int* cells, uint16_t* edges, int* parents);
/* FP64 DMC vertex positions for a grid of the same dims, topology held fixed */
void mdmc_oracle_positions_f64(const void* result, const double* grid, const int dims[3], const double origin[3],
                               const double spacing[3], double iso, double* out);
/* FP64 gradient of sum(dLdpos . positions) (3 per final vertex) with respect to
 * the grid samples, added to out */
void mdmc_oracle_backward(const void* result, const double* grid, const int dims[3], const double spacing[3],
                          double iso, const double* dLdpos, double* out);
/* refineGrid as a linear map in FP64 (coarse dims in), and its adjoint (added to din) */
void mdmc_oracle_refine_f64(const double* in, const int dims[3], int r, int pad, double* out);
void mdmc_oracle_refine_backward(const double* dout, const int dims[3], int r, int pad, double* din);

/* 1 if Marching Cubes case c takes the asymptotic-decider path. */
int mdmc_oracle_case_ambiguous(int c);

#ifdef __cplusplus
}
#endif
