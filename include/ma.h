/*
 * ma.h -- C ABI of the GB300 semi-discrete optimal-transport engine.
 *
 * Drop-in boundary for the hot path of MongeAmpere++ (mrgt/MongeAmpere).  Each
 * entry point below replaces one header-only C++ template of the reference and
 * keeps its argument meaning:
 *
 *   ma_kantorovich     MA::kantorovich               include/MA/kantorovich.hpp:35-141
 *   ma_hessian_copy    the SparseMatrix h it fills    include/MA/kantorovich.hpp:137-139
 *   ma_ot_solve        MA::ot_solve + Statistics      include/MA/optimal_transport.hpp:35-39, 89-193
 *   ma_laplacian_solve MA::solve_laplacian_matrix     include/MA/optimal_transport.hpp:41-87
 *   ma_moments         MA::first_moment / second_moment  include/MA/lloyd.hpp:30-123
 *   ma_lloyd           MA::lloyd                      include/MA/lloyd.hpp:126-144
 *   ma_w2_flow         the iterated solve + centroid step of tests/test_zeldovich.cpp:99-119
 *   ma_pieces          MA::voronoi_triangulation_intersection
 *                                                     include/MA/voronoi_triangulation_intersection.hpp:315-343
 *   ma_ot_solve_batch  no counterpart in the reference: many problems, solved concurrently
 *   ma_draw_laguerre   MA::draw_laguerre_diagram        include/MA/rasterization.hpp:516-547
 *   ma_polygon_cells   MA::voronoi_polygon_intersection, for every site at once
 *                                                     include/MA/voronoi_polygon_intersection.hpp:153-188
 *   ma_kantorovich_vjp no counterpart in the reference: the adjoint of ma_kantorovich
 *                      and ma_moments (vector-Jacobian product)
 *   ma_mesh_create_image image_to_pl_function           include/MA/functions.hpp:82-120
 *   ma_mesh_create_*   the density: a triangulation plus one linear function per
 *                      face (include/MA/functions.hpp:55-120,
 *                      include/CGAL/Triangulation_incremental_builder_2.h:27-80)
 *
 * Conventions
 *   - Sites are passed as two arrays x[n], y[n]: for the reference's N x 2
 *     column-major Eigen matrix X, x = X.data() and y = X.data() + N.
 *   - Every pointer argument is caller-owned; `mem` says whether the arrays live in
 *     host memory (MA_MEM_HOST, copied through the context's pinned staging) or in
 *     device memory of the context's GPU (MA_MEM_DEVICE, used in place).
 *   - Every call returns an ma_status; the reference reports errors only through
 *     assert() and stderr (optimal_transport.hpp:49-58, 137-148).
 *   - A context owns one CUDA stream and all scratch memory.  Calls on one context
 *     must not overlap; separate contexts may be used from separate threads.
 */
#ifndef MA_H
#define MA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ma_status {
    MA_OK = 0,
    MA_ERR_INVALID_ARGUMENT = 1,
    MA_ERR_NO_DEVICE = 2,       /* no CUDA device, or the device is not sm_103 */
    MA_ERR_CUDA = 3,            /* a CUDA runtime call failed (see ma_ctx_last_error) */
    MA_ERR_OUT_OF_MEMORY = 4,
    MA_ERR_CAPACITY = 5,        /* a cell needed more polygon vertices than any kernel holds */
    MA_ERR_EXACT_OVERFLOW = 6,  /* an exact predicate ran out of expansion capacity */
    MA_EMPTY_CELL = 7,          /* ot_solve: a Laguerre cell is empty at the start
                                   (optimal_transport.hpp:137-148) */
    MA_LINESEARCH_FAIL = 8,     /* ot_solve: the step fell below 2^-40 */
    MA_MAXITER = 9,             /* ot_solve: maxiter reached before the stop rule held */
    MA_ERR_BUFFER_TOO_SMALL = 10,
    MA_CG_NOCONV = 11           /* a linear solve stopped at its iteration cap, or broke down (p.Hp <= 0),
                                   before its relative residual reached rtol; the output holds the
                                   last iterate (the reference's SimplicialLLT has no such state; its
                                   residual check, optimal_transport.hpp:67-79, falls back to SPQR) */
} ma_status;

typedef enum ma_mem { MA_MEM_HOST = 0, MA_MEM_DEVICE = 1 } ma_mem;

typedef enum ma_precision {
    MA_FP64 = 0,   /* the reference's arithmetic: FP64 integrals, exact combinatorics */
    MA_MIXED = 1   /* FP32 piece integrals (from FP32 vertex positions), summed per cell in FP64;
                      combinatorics still certified / exact.  ma_ot_solve iterates on these
                      evaluations, then finishes on FP64 evaluations: its stopping test and
                      result are those of the FP64 masses; the linear solves stay FP64 */
} ma_precision;

typedef enum ma_stop_rule {
    MA_STOP_GRAD_NORM = 0,   /* the reference's rule: |m - nu|_2 < eps_g (optimal_transport.hpp:150) */
    MA_STOP_MAX_REL = 1      /* max_i |m_i - nu_i| / nu_i <= eps_g */
} ma_stop_rule;

typedef struct ma_ctx ma_ctx;
typedef struct ma_mesh ma_mesh;

/* ------------------------------------------------------------------ context */
const char* ma_status_string(ma_status s);
ma_status ma_ctx_create(int device, ma_ctx** out);
void ma_ctx_destroy(ma_ctx* ctx);
/* Use `stream` (a cudaStream_t) instead of the context's own stream. */
ma_status ma_ctx_set_stream(ma_ctx* ctx, void* stream);
const char* ma_ctx_last_error(const ma_ctx* ctx);
/* Number of kernel launches the context has issued since it was created. */
int64_t ma_ctx_launch_count(const ma_ctx* ctx);

/* Device-time profile of the main kernels (CUDA events around each launch). */
typedef struct ma_profile {
    double cells_ms;          /* Laguerre cells: site-tree search and clipping (stage 1) */
    int64_t cells_launches;
    double pieces_ms;         /* cell-triangle pieces: clipping and FP64 integrals (stage 2) */
    int64_t pieces_launches;
    double cells_large_ms;    /* large-capacity pass */
    int64_t cells_large_launches;
    double bounds_ms;         /* site-tree bounds, once per evaluation */
    int64_t bounds_launches;
    double pcg_ms;            /* cooperative CG kernel */
    int64_t pcg_launches;
    int64_t pcg_iters;
    int64_t large_sites;      /* sites redone by the large-capacity pass */
    int64_t search[6];        /* stage-1 totals: tree nodes popped, node bounds tested, nodes
                                 pruned, candidate sites clipped against, clips that cut,
                                 final neighbours */
    int64_t amg_fallbacks;    /* Newton solves whose multigrid setup met a coarse row beyond its
                                 capacity and ran with the diagonal preconditioner */
    double amg_setup_ms;      /* multigrid hierarchy: fine matrix, aggregation, Galerkin levels */
    int64_t amg_levels;       /* levels of the last hierarchy */
    int64_t mixed[4];         /* mixed-precision evaluations: pieces integrated, cells redone in
                                 FP64 (their certified FP32 mass error above 2^-12), radical-axis
                                 edges, edges integrated in FP64 */
} ma_profile;
/* enable != 0: reset the profile and start recording; 0: stop. */
ma_status ma_ctx_profile(ma_ctx* ctx, int enable);
ma_status ma_ctx_profile_read(const ma_ctx* ctx, ma_profile* out);

/* --------------------------------------------------------------------- mesh */
/* Tensor-product grid: vertex (i, j) at (gx[i], gy[j]) with value values[j*nx + i];
 * square (i, j) is split along its (i,j)-(i+1,j+1) diagonal.  Host arrays. */
ma_status ma_mesh_create_grid(ma_ctx* ctx, int nx, int ny, const double* gx, const double* gy,
                              const double* values, ma_mesh** out);
/* Explicit triangulation (nv vertices, nt counter-clockwise triangles).  Host arrays. */
ma_status ma_mesh_create_triangles(ma_ctx* ctx, int nv, const double* vx, const double* vy,
                                   const double* values, int nt, const int32_t* tri, ma_mesh** out);
/* image_to_pl_function (functions.hpp:82-120): the density of a grey image,
 * pixels[height][width] (rows top first, values 0..255, as CImg's image(x, y)), on a
 * width x height vertex grid of [-1, 1]^2 with vertex values pixel / 255 + 1e-3; the
 * total mass is ma_mesh_total_mass.  The reference triangulates the grid points with
 * CGAL's Delaunay triangulation, whose split of each (co-circular) square is CGAL's
 * choice; here every square is split along its (i, j)-(i+1, j+1) diagonal. */
ma_status ma_mesh_create_image(ma_ctx* ctx, int width, int height, const double* pixels, ma_mesh** out);
/* New vertex values for an existing mesh (same geometry): values[nx*ny] for a grid,
 * values[nv] for a triangle mesh, in host or device memory.  The density is a
 * differentiable input of ma_kantorovich_vjp; this updates it without rebuilding the
 * mesh's bins. */
ma_status ma_mesh_set_values(ma_ctx* ctx, ma_mesh* mesh, const double* values, ma_mem mem);
void ma_mesh_destroy(ma_mesh* mesh);
/* Integral of the density (the value image_to_pl_function returns, functions.hpp:116-119). */
ma_status ma_mesh_total_mass(const ma_mesh* mesh, double* out);

/* -------------------------------------------------------------- kantorovich */
/* One evaluation of MA::kantorovich: value = sum_i (w_i m_i - int_{Lag_i} rho |x - x_i|^2),
 * g[i] = m_i = int_{Lag_i} rho, and the Hessian H (kept in the context; read it with
 * ma_hessian_copy).  *nnz receives the number of stored Hessian entries. */
ma_status ma_kantorovich(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                         const double* w, ma_mem mem, ma_precision prec, double* value, double* g,
                         int64_t* nnz);
/* The Hessian of the last ma_kantorovich call in CSR form: rowptr[n+1], col[nnz] (sorted,
 * diagonal included), val[nnz].  Since H is symmetric this is also the reference's
 * column-major SparseMatrix storage (outer = rowptr, inner = col). */
ma_status ma_hessian_copy(ma_ctx* ctx, int32_t* rowptr, int32_t* col, double* val, ma_mem mem);

/* ------------------------------------------------------------------ solver */
typedef enum ma_precond {
    MA_PRECOND_MULTIGRID = 0, /* one V-cycle of an aggregation multigrid (default) */
    MA_PRECOND_JACOBI = 1     /* diagonal scaling */
} ma_precond;

typedef enum ma_init {
    MA_INIT_GIVEN = 0,      /* start from w_inout (the reference's behaviour; zeros = its empty start) */
    MA_INIT_MULTISCALE = 1, /* coarse-to-fine initial guess: sites aggregated by 8 in Morton order
                               down to ~4,000, each level solved to 1e-2 relative from its parent's
                               weights (no counterpart in the reference, whose ot_solve takes the
                               initial guess as an argument); for sites near a uniform spread */
    MA_INIT_CONTINUATION = 2 /* continuation in the target masses from those of w_inout: stages
                               nu_t = m(w_in) + t (nu - m(w_in)), no cell's target changing by more
                               than 2x between stages, each the reference's damped Newton to 1e-1
                               relative (at most 5 * maxiter steps), the last one to the caller's
                               rule; no counterpart in the reference.  For sites far from equilibrium
                               (clustered sites), where the damped Newton from w_inout stalls */
} ma_init;

typedef struct ma_solve_opts {
    double eps_g;          /* stop threshold (reference default 1e-7) */
    int64_t maxiter;       /* Newton iterations (reference default 100) */
    int stop_rule;         /* ma_stop_rule */
    int precision;         /* ma_precision */
    int verbose;           /* print the reference's per-iteration line to stderr */
    double cg_rtol;        /* relative residual of the preconditioned CG; 0 (default): inexact Newton
                              with the forcing term 1e-2 */
    int64_t cg_maxiter;    /* CG iteration cap (0: default 20000) */
    int precond;           /* ma_precond: CG preconditioner of the Newton step */
    int init;              /* ma_init: initial guess */
} ma_solve_opts;

typedef struct ma_stats {
    size_t niter;                /* Statistics::niter (optimal_transport.hpp:35-39) */
    size_t neval;                /* Statistics::neval */
    size_t cg_iters;             /* total CG iterations */
    size_t linesearch_halvings;
    double grad_norm;            /* |m - nu|_2 at exit */
    double max_rel_err;          /* max_i |m_i - nu_i| / nu_i at exit */
    double value;                /* Kantorovich value minus <nu, w> at exit (NaN after
                                    MA_LINESEARCH_FAIL) */
    double t_eval_ms;            /* device time spent in Laguerre evaluations */
    double t_linsolve_ms;        /* device time spent in linear solves */
    size_t neval_fp64;           /* evaluations with FP64 integrals (all of them unless precision
                                    is MA_MIXED) */
    size_t cg_noconv;            /* Newton steps whose CG stopped at cg_maxiter (or broke down) before
                                    its residual met the forcing term: the step went on with the
                                    unconverged direction, checked by the line search as usual */
} ma_stats;

void ma_solve_opts_default(ma_solve_opts* o);
/* Damped Newton (Kitagawa-Merigot-Thibert) on m(w) = nu.  w_inout holds the initial
 * guess on entry (pass all zeros for the reference's empty-vector start) and the
 * solution on exit; the gauge is w[n-1] fixed, as solve_laplacian_matrix does. */
ma_status ma_ot_solve(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                      const double* nu, double* w_inout, ma_mem mem, const ma_solve_opts* opts,
                      ma_stats* stats);
/* ------------------------------------------------------------------- batch */
/* Many independent problems (no counterpart in the reference, which solves one per
 * MA::ot_solve call).  Each problem has its own mesh (created on any context of the
 * same device), sites, target masses and weights (initial guess in, solution out);
 * every array of the batch is in `mem`.  The problems are solved by `workers`
 * contexts (one CUDA stream and one host thread each) taking them in order; kernels of
 * different problems run concurrently.  workers = 0 autotunes the count (4 to 64) by
 * solving copies of the batch's median problem (kept in the context for later calls);
 * *workers_used (nullable) receives the count used.  Each problem is solved by
 * ma_ot_solve (status and statistics are its); a worker's CG uses a share of the GPU,
 * so results agree with separate calls to the solver's tolerance, not to the last bit.
 * The call returns MA_OK unless a CUDA or argument error stopped a worker.  The
 * workers' streams share the device's hardware work queues: a process that batches
 * should set CUDA_DEVICE_MAX_CONNECTIONS=32 before it creates its CUDA context (the
 * default, 8, serialises the streams onto 8 queues; 512 mixed problems of 500-50,000
 * sites went from 188 to 236 problems/s with 32). */
typedef struct ma_problem {
    const ma_mesh* mesh;
    int64_t n;
    const double* x;
    const double* y;
    const double* nu;
    double* w;
    ma_status status; /* out */
    ma_stats stats;   /* out */
} ma_problem;
ma_status ma_ot_solve_batch(ma_ctx* ctx, ma_problem* problems, int64_t count, ma_mem mem,
                            const ma_solve_opts* opts, int workers, int* workers_used);

/* A W2 gradient-flow / Lloyd driver (tests/test_zeldovich.cpp:99-119, lloyd.hpp:126-144):
 * `steps` times, an OT solve of the sites to `nu` (ma_ot_solve with `opts`, warm-started
 * from the previous weights, or from zero weights when a moved site's cell is empty
 * there), the cells' centroids c (int rho x / int rho), then
 * x <- x + tau (x - c) (tau = 0.03 is the reference's Zel'dovich-type step, tau = -1 a
 * Lloyd step).  x, y and w are updated in place; *stats sums the solves.  The
 * reference restarts every solve from zero weights and uses the cells' geometric
 * barycentres; for a constant density the two barycentres agree. */
ma_status ma_w2_flow(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, double* x, double* y, const double* nu,
                     double* w, ma_mem mem, int64_t steps, double tau, const ma_solve_opts* opts,
                     ma_stats* stats);

/* Newton direction of solve_laplacian_matrix: solve H[:n-1,:n-1] d = g[:n-1], d[n-1] = 0,
 * for the Hessian of the last ma_kantorovich call.  Returns the CG iteration count in *iters;
 * MA_CG_NOCONV (with d the last iterate) when the CG stopped before |r| <= rtol |g|.
 * rtol <= 0 means 1e-10; maxiter <= 0 means 20000 (larger values are capped at INT_MAX). */
ma_status ma_laplacian_solve(ma_ctx* ctx, const double* g, double* d, ma_mem mem, double rtol,
                             int64_t maxiter, int64_t* iters);

/* Newton linear solve that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot let a library allocate device memory -- applications whose
 * own pool or arena owns all device memory, and latency-critical loops that cannot
 * afford the device-wide synchronisation of cudaMalloc / cudaFree.  It solves
 * H[:n-1,:n-1] d = g[:n-1], d[n-1] = 0 (the system of ma_laplacian_solve) for a CSR
 * Hessian the caller passes in; rowptr, col, val, g and d are device memory of the
 * current device, `stream` is a cudaStream_t (NULL: the default stream), *iters (host)
 * receives the CG iteration count.  rtol <= 0 means 1e-10; maxiter <= 0 means 20000 and
 * larger values are capped at INT_MAX.  The call returns MA_CG_NOCONV, with d holding the
 * last iterate, when the CG stopped at maxiter (or broke down) before |r| <= rtol |g|.
 *  - The CG work vectors live in one fixed device array of the library (10.1 MB, held
 *    by every GPU that loads the library until the process exits); n is limited to
 *    262,144 and larger systems return MA_ERR_BUFFER_TOO_SMALL.
 *  - The first call on a device looks up that array's address, so make that first call
 *    before any stream capture begins.
 *  - Every call shares the array: calls that overlap on the GPU (from several threads
 *    or streams) race and corrupt each other's result. */
ma_status ma_laplacian_solve_static(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                                    const double* g, double* d, double rtol, int64_t maxiter, int64_t* iters,
                                    void* stream);

/* ------------------------------------------------------------------ pieces */
/* MA::voronoi_triangulation_intersection (voronoi_triangulation_intersection.hpp:
 * 315-343): every non-empty intersection of a Laguerre cell with a mesh triangle, as
 * a convex polygon.  The reference hands each piece to a callback out(polygon, face,
 * vertex); here ma_pieces computes them all on the device and returns their number
 * and their total vertex count, and ma_pieces_copy fills (each pointer nullable):
 *   site[np]    the cell's site (original index)     -- the reference's Vertex_handle
 *   tri[np]     the mesh triangle (grid: 2 (j (nx-1) + i) + t, the explicit
 *               triangulation's order; triangle mesh: its index) -- the Face_handle
 *   off[np+1]   first vertex of each piece; off[np] = nverts
 *   xy[2 nv]    polygon vertices, counter-clockwise, absolute (x, y)
 *   edge[nv]    the edge from vertex k to vertex k+1: the neighbouring site whose
 *               radical axis it lies on (original index; the reference's EDGE_DT), or
 *               -1-e for edge e (v_e -> v_e+1) of the triangle (EDGE_T)
 * Pieces are ordered by cell (in the site index's Morton order), then by triangle.
 * Cells of more than 48 neighbours, or whose clips meet exact ties (lattice sites,
 * bisectors through mesh vertices), are listed by a one-thread-per-cell pass with exact
 * predicates; MA_ERR_CAPACITY only for a cell beyond its 256 slots. */
ma_status ma_pieces(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                    const double* w, ma_mem mem, int64_t* npieces, int64_t* nverts);
ma_status ma_pieces_copy(ma_ctx* ctx, int32_t* site, int32_t* tri, int64_t* off, double* xy, int32_t* edge,
                         ma_mem mem);

/* MA::voronoi_polygon_intersection (voronoi_polygon_intersection.hpp:153-188), run
 * for every site: the Laguerre cell of each site (weights w, or the Voronoi cell when
 * w is null) intersected with the polygon (px[e], py[e]), e < k, 3 <= k <= 64 -- the
 * reference's polygon P, here in host memory.  P need not be convex: as in the
 * reference's Pgon_intersector (:116-149) it is clipped by the half-planes of the
 * site's neighbours, so a non-convex P can give a polygon with bridging edges of zero
 * area.  ma_polygon_cells returns the total vertex count; ma_polygon_cells_copy
 * fills (each pointer nullable):
 *   off[n+1]    first vertex of site i's polygon (original order); off[n] = nverts;
 *               an empty intersection has off[i] = off[i+1]
 *   xy[2 nv]    vertices (x, y), in P's orientation; P's own corners are copied exactly
 *   edge[nv]    the edge from vertex k to vertex k+1: the neighbouring site whose
 *               radical axis it lies on (original index; the reference's DELAUNAY
 *               edge), or -1-e for edge e (P_e -> P_e+1) of P (the reference's POLYGON
 *               edge).
 * The predicates are exact (filters with an exact fallback); MA_ERR_CAPACITY when a
 * cell needs more than 256 slots or vertices. */
ma_status ma_polygon_cells(ma_ctx* ctx, int64_t n, const double* x, const double* y, const double* w,
                           const double* px, const double* py, int k, ma_mem mem, int64_t* nverts);
ma_status ma_polygon_cells_copy(ma_ctx* ctx, int64_t* off, double* xy, int32_t* edge, ma_mem mem);

/* MA::draw_laguerre_diagram (rasterization.hpp:516-547): every piece rasterised with
 * exact pixel coverage into image[height][width][channels] (row y = 0 first; pixel
 * (i, j) covers [x0 + i dx, x0 + (i+1) dx] x [y0 + j dy, y0 + (j+1) dy] with
 * dx = (x1 - x0) / width), adding cover * (mean of the density at the piece's
 * vertices) * colors[site][channel] -- the reference's put_pixel(x, y, cover * ff *
 * color); the image is added to (zero it for a plain drawing).  colors[n][channels],
 * channels 1..16; image and colors in `mem`. */
ma_status ma_draw_laguerre(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                           const double* w, const double* colors, int channels, double x0, double y0,
                           double x1, double y1, int width, int height, double* image, ma_mem mem);

/* ----------------------------------------------------------------- adjoint */
/* Vector-Jacobian product of (value, mass[n], first[2n]) -- the Kantorovich value
 * sum_i (w_i m_i - int_{cell i} rho |x - x_i|^2), the cell masses and the first
 * moments int_{cell i} rho x of ma_moments -- with respect to the site positions,
 * the weights and the density's vertex values.  No counterpart in the reference (it
 * has no derivatives beyond the Hessian in w); this is for gradient-based callers
 * (W2 gradient flows, Lloyd-type descent, learning pipelines) that differentiate
 * through the transport.
 *   cot_value           cotangent of the value
 *   cot_mass[n]         cotangents of the masses (NULL: zero)
 *   cot_first[2n]       cotangents of the first moments, (x, y) per site (NULL: zero)
 *   grad_x, grad_y, grad_w [n]  receive the gradients with respect to the sites and weights
 *   grad_rho            receives the gradient with respect to the mesh's vertex values
 *                       (grid: nx * ny, row-major like the values; triangles: nv), or NULL
 *   prec                MA_FP64, or MA_MIXED: the pieces' integrals in FP32 about a point of
 *                       each cell (the mixed evaluation's), moved to the site-relative moments
 *                       and summed per cell in FP64
 * Cells with more than 48 neighbours, or whose pieces need exact predicates, are not
 * handled (MA_ERR_CAPACITY).  grad_rho is accumulated with atomics: its last bits may
 * differ from run to run; the other gradients are reproducible. */
ma_status ma_kantorovich_vjp(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                             const double* w, ma_mem mem, ma_precision prec, double cot_value, const double* cot_mass,
                             const double* cot_first, double* grad_x, double* grad_y, double* grad_w,
                             double* grad_rho);

/* --------------------------------------------------------- moments / Lloyd */
/* mass[n]; first[2n] = (int rho x, int rho y) per site; second[3n] (nullable) =
 * (int rho x^2, int rho y^2, int rho x y) per site. */
ma_status ma_moments(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                     const double* w, ma_mem mem, double* mass, double* first, double* second);
/* mass[n] and centroids[2n] (first moments divided by mass). */
ma_status ma_lloyd(ma_ctx* ctx, const ma_mesh* mesh, int64_t n, const double* x, const double* y,
                   const double* w, ma_mem mem, double* mass, double* centroids);

#ifdef __cplusplus
}
#endif

#endif /* MA_H */
