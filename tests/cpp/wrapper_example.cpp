// A MongeAmpere++-style caller of the C++ wrapper (include/MA/gb300.hpp): the
// reference's entry points with their argument order, on a 3 x 3 grid density.
// Exit status: 0 success, 3 an MA::Error (printed), 4 a wrong result.
#include <MA/gb300.hpp>

#include <cmath>
#include <cstdio>

struct Mat {  // the N x 2 matrix interface the templates use (Eigen::MatrixXd works too)
    std::vector<double> d;
    int64_t n = 0;
    int64_t rows() const { return n; }
    int64_t cols() const { return 2; }
    double operator()(int64_t i, int64_t j) const { return d[2 * i + j]; }
    double& operator()(int64_t i, int64_t j) { return d[2 * i + j]; }
    void resize(int64_t r, int64_t) { n = r, d.resize(2 * r); }
};
struct Vec {
    std::vector<double> d;
    int64_t size() const { return (int64_t)d.size(); }
    int64_t rows() const { return size(); }
    double operator[](int64_t i) const { return d[i]; }
    double& operator[](int64_t i) { return d[i]; }
    void resize(int64_t n) { d.resize(n); }
};

int main()
{
    std::vector<double> g{0.0, 0.5, 1.0}, v(9, 1.0);
    try {
        MA::Density rho = MA::Density::grid(g, g, v);
        Mat X;
        X.d = {0.2, 0.3, 0.7, 0.6, 0.4, 0.8};
        X.n = 3;
        Vec w{{0.0, 0.0, 0.0}}, gr, masses{{1.0 / 3, 1.0 / 3, 1.0 / 3}}, x;
        MA::SparseCSR h;
        MA::kantorovich(rho, X, w, gr, h);
        double tot = gr[0] + gr[1] + gr[2];
        MA::Statistics stats;
        MA::ot_solve(rho, X, masses, x, 1e-12, 50, false, &stats);
        MA::kantorovich(rho, X, x, gr, h);
        double err = 0;
        for (int i = 0; i < 3; i++) err = std::fmax(err, std::fabs(gr[i] - 1.0 / 3));
        double area = 0;
        int np = 0;
        MA::voronoi_triangulation_intersection(rho, X, x, [&](const MA::Piece& p) {
            np++;
            const size_t k = p.polygon.size();
            for (size_t a = 0; a < k; a++) {
                const auto& P = p.polygon[a];
                const auto& Q = p.polygon[(a + 1) % k];
                area += 0.5 * (P.first * Q.second - Q.first * P.second);
            }
        });
        // the cells clipped to the unit square add up to its area
        MA::Polygon sq{{0.0, 0.0}, {1.0, 0.0}, {1.0, 1.0}, {0.0, 1.0}};
        double parea = 0;
        for (const MA::Polygon& R : MA::voronoi_polygon_intersection(sq, X, x)) {
            const size_t k = R.size();
            for (size_t a = 0; a < k; a++)
                parea += 0.5 * (R[a].first * R[(a + 1) % k].second - R[(a + 1) % k].first * R[a].second);
        }
        std::printf("total mass %.15g, solve error %.3g after %zu Newton steps, %d pieces of area %.15g, "
                    "clipped cells of area %.15g\n",
                    tot, err, stats.niter, np, area, parea);
        if (std::fabs(tot - 1.0) > 1e-12 || err > 1e-12 || std::fabs(area - 1.0) > 1e-12 || h.nonZeros() != 9 ||
            std::fabs(parea - 1.0) > 1e-12)
            return 4;
    } catch (const MA::Error& e) {
        std::printf("MA::Error: %s\n", e.what());
        return 3;
    }
    return 0;
}
