// MA/gb300.hpp -- the reference's C++ entry points over the GB300 C ABI.
//
// A MongeAmpere++ caller keeps its call sites: MA::kantorovich, MA::ot_solve,
// MA::first_moment, MA::second_moment, MA::lloyd, MA::solve_laplacian_matrix,
// MA::voronoi_triangulation_intersection, MA::voronoi_polygon_intersection keep
// their names, argument order and argument meaning (include/MA/kantorovich.hpp:35-42,
// include/MA/optimal_transport.hpp:35-39, 41-44, 89-99, include/MA/lloyd.hpp:30-36,
// 71-78, 126-132).  The triangulation + per-face linear functions of the reference
// become one `MA::Density` (a device copy of the mesh, built once), and the Eigen
// types become any types that provide what the templates use:
//
//   Matrix  X   : rows(), cols(), operator()(i, j) (an N x 2 Eigen::MatrixXd works)
//   Vector  w   : rows() / size(), operator[](i) / operator()(i), resize(n)
//   Sparse  h   : the templates fill a CSR triple through `set_csr(n, rowptr, col, val)`;
//                 MA::SparseCSR below is a ready-made one.  Because H is symmetric the
//                 CSR arrays are also the column-major (CSC) storage Eigen uses.
//
// Host-memory callers only: every array is copied through the context.
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../ma.h"

namespace MA {

struct Error : std::runtime_error {
    ma_status status;
    Error(ma_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(ma_status s, ma_ctx* ctx, const char* what)
{
    if (s != MA_OK) {
        std::string m = std::string(what) + ": " + ma_status_string(s);
        if (ctx) {
            const char* e = ma_ctx_last_error(ctx);
            if (e && *e) m += std::string(" (") + e + ")";
        }
        throw Error(s, m);
    }
}

// one CUDA context of the engine (stream + scratch), created on first use
class Engine {
public:
    explicit Engine(int device = 0) { check(ma_ctx_create(device, &ctx_), nullptr, "ma_ctx_create"); }
    ~Engine() { ma_ctx_destroy(ctx_); }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    ma_ctx* get() const { return ctx_; }
    static Engine& instance()
    {
        static Engine e(0);
        return e;
    }

private:
    ma_ctx* ctx_ = nullptr;
};

// the density: a triangulation with one linear function per face
class Density {
public:
    // tensor-product grid, values[j * nx + i] at (gx[i], gy[j])
    static Density grid(const std::vector<double>& gx, const std::vector<double>& gy,
                        const std::vector<double>& values, Engine& e = Engine::instance())
    {
        Density d;
        d.ctx_ = e.get();
        check(ma_mesh_create_grid(d.ctx_, (int)gx.size(), (int)gy.size(), gx.data(), gy.data(), values.data(),
                                  &d.mesh_),
              d.ctx_, "ma_mesh_create_grid");
        return d;
    }
    // explicit triangulation (what Triangulation_incremental_builder_2 assembles)
    static Density triangles(const std::vector<double>& vx, const std::vector<double>& vy,
                             const std::vector<double>& values, const std::vector<int32_t>& tri,
                             Engine& e = Engine::instance())
    {
        Density d;
        d.ctx_ = e.get();
        check(ma_mesh_create_triangles(d.ctx_, (int)vx.size(), vx.data(), vy.data(), values.data(),
                                       (int)(tri.size() / 3), tri.data(), &d.mesh_),
              d.ctx_, "ma_mesh_create_triangles");
        return d;
    }
    // image_to_pl_function (functions.hpp:82-120): the density of a grey image,
    // pixels[y * width + x] with rows top first and values 0..255 (CImg's image(x, y)),
    // on a width x height vertex grid of [-1, 1]^2 with vertex values pixel / 255 + 1e-3.
    // total_mass() is the value the reference returns.
    static Density image(const std::vector<double>& pixels, int width, int height,
                         Engine& e = Engine::instance())
    {
        if (width < 2 || height < 2 || (int64_t)pixels.size() != (int64_t)width * height)
            throw Error(MA_ERR_INVALID_ARGUMENT, "image_to_pl_function: pixels.size() must be width * height");
        Density d;
        d.ctx_ = e.get();
        check(ma_mesh_create_image(d.ctx_, width, height, pixels.data(), &d.mesh_), d.ctx_, "ma_mesh_create_image");
        return d;
    }
    Density(Density&& o) noexcept : ctx_(o.ctx_), mesh_(o.mesh_) { o.mesh_ = nullptr; }
    ~Density() { ma_mesh_destroy(mesh_); }
    ma_mesh* get() const { return mesh_; }
    ma_ctx* ctx() const { return ctx_; }
    // the value image_to_pl_function returns (functions.hpp:116-119)
    double total_mass() const
    {
        double m = 0;
        check(ma_mesh_total_mass(mesh_, &m), ctx_, "ma_mesh_total_mass");
        return m;
    }

private:
    Density() = default;
    ma_ctx* ctx_ = nullptr;
    ma_mesh* mesh_ = nullptr;
};

// a minimal CSR matrix for the Hessian
struct SparseCSR {
    int64_t n = 0;
    std::vector<int32_t> rowptr, col;
    std::vector<double> val;
    void set_csr(int64_t rows, std::vector<int32_t> rp, std::vector<int32_t> c, std::vector<double> v)
    {
        n = rows;
        rowptr = std::move(rp);
        col = std::move(c);
        val = std::move(v);
    }
    int64_t rows() const { return n; }
    int64_t nonZeros() const { return (int64_t)val.size(); }
};

struct Statistics {  // optimal_transport.hpp:35-39, plus the engine's counters
    size_t niter = 0;
    size_t neval = 0;
    ma_stats full{};
};

namespace detail {
template <class Matrix>
void split_sites(const Matrix& X, std::vector<double>& x, std::vector<double>& y)
{
    const int64_t n = (int64_t)X.rows();
    x.resize(n);
    y.resize(n);
    for (int64_t i = 0; i < n; i++) {
        x[i] = X(i, 0);
        y[i] = X(i, 1);
    }
}
template <class Vector>
std::vector<double> to_vec(const Vector& v, int64_t n)
{
    std::vector<double> r(n);
    for (int64_t i = 0; i < n; i++) r[i] = v[i];
    return r;
}
template <class Vector>
void from_vec(Vector& v, const std::vector<double>& r)
{
    v.resize((int64_t)r.size());
    for (size_t i = 0; i < r.size(); i++) v[i] = r[i];
}
}  // namespace detail

// MA::kantorovich (kantorovich.hpp:35-141): returns the value, fills g (cell masses)
// and h (the Hessian)
template <class Matrix, class Vector, class SparseMatrix>
double kantorovich(const Density& density, const Matrix& X, const Vector& weights, Vector& g, SparseMatrix& h)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n), gg(n);
    double value = 0;
    int64_t nnz = 0;
    check(ma_kantorovich(density.ctx(), density.get(), n, x.data(), y.data(), w.data(), MA_MEM_HOST, MA_FP64,
                         &value, gg.data(), &nnz),
          density.ctx(), "ma_kantorovich");
    std::vector<int32_t> rp(n + 1), col(nnz);
    std::vector<double> val(nnz);
    check(ma_hessian_copy(density.ctx(), rp.data(), col.data(), val.data(), MA_MEM_HOST), density.ctx(),
          "ma_hessian_copy");
    detail::from_vec(g, gg);
    h.set_csr(n, std::move(rp), std::move(col), std::move(val));
    return value;
}

// MA::ot_solve (optimal_transport.hpp:89-193); x is the initial guess and the result
template <class Matrix, class Vector>
void ot_solve(const Density& density, const Matrix& X, const Vector& masses, Vector& x, double eps_g = 1e-7,
              size_t maxiter = 100, bool verbose = true, Statistics* stats = nullptr)
{
    std::vector<double> xs, ys;
    detail::split_sites(X, xs, ys);
    const int64_t n = (int64_t)xs.size();
    std::vector<double> nu = detail::to_vec(masses, n);
    std::vector<double> w(n, 0.0);
    if ((int64_t)x.size() == n) w = detail::to_vec(x, n);
    ma_solve_opts o;
    ma_solve_opts_default(&o);
    o.eps_g = eps_g;
    o.maxiter = (int64_t)maxiter;
    o.verbose = verbose ? 1 : 0;
    ma_stats st{};
    ma_status s = ma_ot_solve(density.ctx(), density.get(), n, xs.data(), ys.data(), nu.data(), w.data(),
                              MA_MEM_HOST, &o, &st);
    if (stats) {
        stats->niter = st.niter;
        stats->neval = st.neval;
        stats->full = st;
    }
    // the reference returns silently when a cell is empty at the start or when
    // maxiter runs out; the weights are still written back in the latter case
    if (s == MA_EMPTY_CELL) return;
    if (s != MA_MAXITER) check(s, density.ctx(), "ma_ot_solve");
    detail::from_vec(x, w);
}

// MA::first_moment (lloyd.hpp:30-69): masses and first moments (N x 2)
template <class Matrix, class Vector>
void first_moment(const Density& density, const Matrix& X, const Vector& weights, Vector& masses,
                  Matrix& centroids)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n), m(n), f(2 * n);
    check(ma_moments(density.ctx(), density.get(), n, x.data(), y.data(), w.data(), MA_MEM_HOST, m.data(),
                     f.data(), nullptr),
          density.ctx(), "ma_moments");
    detail::from_vec(masses, m);
    centroids.resize(n, 2);
    for (int64_t i = 0; i < n; i++) {
        centroids(i, 0) = f[2 * i];
        centroids(i, 1) = f[2 * i + 1];
    }
}

// MA::second_moment (lloyd.hpp:71-123): masses, first moments, inertia (xx, yy, xy)
template <class Matrix, class Vector>
void second_moment(const Density& density, const Matrix& X, const Vector& weights, Vector& masses,
                   Matrix& centroids, Matrix& inertia)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n), m(n), f(2 * n), s(3 * n);
    check(ma_moments(density.ctx(), density.get(), n, x.data(), y.data(), w.data(), MA_MEM_HOST, m.data(),
                     f.data(), s.data()),
          density.ctx(), "ma_moments");
    detail::from_vec(masses, m);
    centroids.resize(n, 2);
    inertia.resize(n, 3);
    for (int64_t i = 0; i < n; i++) {
        centroids(i, 0) = f[2 * i];
        centroids(i, 1) = f[2 * i + 1];
        for (int k = 0; k < 3; k++) inertia(i, k) = s[3 * i + k];
    }
}

// MA::lloyd (lloyd.hpp:126-144): masses and centroids
template <class Matrix, class Vector>
void lloyd(const Density& density, const Matrix& X, const Vector& weights, Vector& masses, Matrix& centroids)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n), m(n), c(2 * n);
    check(ma_lloyd(density.ctx(), density.get(), n, x.data(), y.data(), w.data(), MA_MEM_HOST, m.data(), c.data()),
          density.ctx(), "ma_lloyd");
    detail::from_vec(masses, m);
    centroids.resize(n, 2);
    for (int64_t i = 0; i < n; i++) {
        centroids(i, 0) = c[2 * i];
        centroids(i, 1) = c[2 * i + 1];
    }
}

// MA::voronoi_triangulation_intersection (voronoi_triangulation_intersection.hpp:
// 315-343): calls out(polygon, triangle, site) for every non-empty intersection of a
// Laguerre cell with a mesh triangle.  polygon is a std::vector of (x, y) pairs,
// counter-clockwise; triangle is the mesh triangle's index (the Face_handle), site
// the site's index (the Vertex_handle); edge[k] labels polygon edge k -> k+1: the
// neighbouring site, or -1-e for edge e of the triangle.
struct Piece {
    int32_t site = 0, triangle = 0;
    std::vector<std::pair<double, double>> polygon;
    std::vector<int32_t> edge;
};

template <class Matrix, class Vector, class Out>
void voronoi_triangulation_intersection(const Density& density, const Matrix& X, const Vector& weights, Out&& out)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n);
    int64_t np = 0, nv = 0;
    check(ma_pieces(density.ctx(), density.get(), n, x.data(), y.data(), w.data(), MA_MEM_HOST, &np, &nv),
          density.ctx(), "ma_pieces");
    std::vector<int32_t> site(np), tri(np), edge(nv);
    std::vector<int64_t> off(np + 1);
    std::vector<double> xy(2 * nv);
    check(ma_pieces_copy(density.ctx(), site.data(), tri.data(), off.data(), xy.data(), edge.data(), MA_MEM_HOST),
          density.ctx(), "ma_pieces_copy");
    Piece p;
    for (int64_t k = 0; k < np; k++) {
        p.site = site[k];
        p.triangle = tri[k];
        p.polygon.clear();
        p.edge.clear();
        for (int64_t v = off[k]; v < off[k + 1]; v++) {
            p.polygon.emplace_back(xy[2 * v], xy[2 * v + 1]);
            p.edge.push_back(edge[v]);
        }
        out(p);
    }
}

// MA::voronoi_polygon_intersection (voronoi_polygon_intersection.hpp:153-188), for
// every site at once: result[i] is the Laguerre cell of site i (weights w) clipped to
// the polygon P, a sequence of (x, y) corners (3 to 64 of them); an empty result when
// the cell misses P.  The reference takes one Vertex_handle of a triangulation per
// call and returns one Polygon; the triangulation here is implicit in the sites and
// weights.  Zero weights give the Delaunay case (Voronoi cells).
using Polygon = std::vector<std::pair<double, double>>;

template <class Matrix, class Vector>
std::vector<Polygon> voronoi_polygon_intersection(const Polygon& P, const Matrix& X, const Vector& weights,
                                                  Engine& e = Engine::instance())
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    std::vector<double> w = detail::to_vec(weights, n), px, py;
    for (const auto& c : P) {
        px.push_back(c.first);
        py.push_back(c.second);
    }
    int64_t nv = 0;
    check(ma_polygon_cells(e.get(), n, x.data(), y.data(), w.data(), px.data(), py.data(), (int)P.size(),
                           MA_MEM_HOST, &nv),
          e.get(), "ma_polygon_cells");
    std::vector<int64_t> off(n + 1);
    std::vector<double> xy(2 * nv);
    check(ma_polygon_cells_copy(e.get(), off.data(), xy.data(), nullptr, MA_MEM_HOST), e.get(),
          "ma_polygon_cells_copy");
    std::vector<Polygon> r((size_t)n);
    for (int64_t i = 0; i < n; i++)
        for (int64_t v = off[i]; v < off[i + 1]; v++) r[(size_t)i].emplace_back(xy[2 * v], xy[2 * v + 1]);
    return r;
}

// MA::draw_laguerre_diagram (rasterization.hpp:516-547): every piece of every Laguerre
// cell rasterised with exact pixel coverage into a height x width x channels image
// (row-major, row 0 first), pixel (i, j) covering [x0 + i dx, x0 + (i+1) dx] x
// [y0 + j dy, y0 + (j+1) dy] with dx = (x1 - x0) / w, dy = (y1 - y0) / h; each piece adds
// cover * (mean density at its vertices) * colors[site][channel].  colors holds n *
// channels values, site-major.
template <class Matrix, class Vector>
std::vector<double> draw_laguerre_diagram(const Density& density, const Matrix& X, const Vector& weights,
                                          const std::vector<double>& colors, int channels, double x0, double y0,
                                          double x1, double y1, size_t w, size_t h)
{
    std::vector<double> x, y;
    detail::split_sites(X, x, y);
    const int64_t n = (int64_t)x.size();
    if (channels < 1 || (int64_t)colors.size() != n * channels)
        throw Error(MA_ERR_INVALID_ARGUMENT, "draw_laguerre_diagram: colors.size() must be n * channels");
    std::vector<double> wv = detail::to_vec(weights, n), image(w * h * (size_t)channels, 0.0);
    check(ma_draw_laguerre(density.ctx(), density.get(), n, x.data(), y.data(), wv.data(), colors.data(), channels,
                           x0, y0, x1, y1, (int)w, (int)h, image.data(), MA_MEM_HOST),
          density.ctx(), "ma_draw_laguerre");
    return image;
}

// The reference's form, with one scalar colour per site and a put_pixel(x, y, value)
// callback: the image is computed as above and put_pixel is called once per pixel
// with the sum of the pieces' contributions to it (the reference calls it once per
// piece and pixel, so a put_pixel that adds gives the same image); pixels that no
// piece covers are not visited.
template <class Matrix, class Vector, class ColorVector, class PutPixel>
void draw_laguerre_diagram(const Density& density, const Matrix& X, const Vector& weights, const ColorVector& colors,
                           double x0, double y0, double x1, double y1, size_t w, size_t h, PutPixel put_pixel)
{
    const int64_t n = (int64_t)X.rows();
    const std::vector<double> img =
        draw_laguerre_diagram(density, X, weights, detail::to_vec(colors, n), 1, x0, y0, x1, y1, w, h);
    for (size_t j = 0; j < h; j++)
        for (size_t i = 0; i < w; i++)
            if (img[j * w + i] != 0.0) put_pixel((int)i, (int)j, img[j * w + i]);
}

// MA::solve_laplacian_matrix (optimal_transport.hpp:41-87) for the Hessian of the
// last kantorovich call on `density`'s engine: d[n-1] = 0
template <class Vector>
Vector solve_laplacian_matrix(const Density& density, const Vector& g)
{
    const int64_t n = (int64_t)g.size();
    std::vector<double> gg = detail::to_vec(g, n), d(n);
    int64_t it = 0;
    const ma_status s = ma_laplacian_solve(density.ctx(), gg.data(), d.data(), MA_MEM_HOST, 1e-12, 0, &it);
    // the reference warns and goes on when its Cholesky residual is large
    // (optimal_transport.hpp:67-79); so does this wrapper when the CG stops early
    if (s == MA_CG_NOCONV)
        std::fprintf(stderr, "WARNING: in solve_laplacian_matrix: %s\n", ma_status_string(s));
    else
        check(s, density.ctx(), "ma_laplacian_solve");
    Vector r;
    detail::from_vec(r, d);
    return r;
}

}  // namespace MA
