// The C++ wrapper's image density and Laguerre-cell drawing (include/MA/gb300.hpp):
// MA::Density::image (image_to_pl_function) and both forms of
// MA::draw_laguerre_diagram.  A white image gives the constant density 1 + 1e-3 on
// [-1, 1]^2, so the drawn pixels (colour 1, exact coverage) add up to the total mass
// over the pixel area, whatever the cells.
// Exit status: 0 success, 3 an MA::Error (printed), 4 a wrong result.
#include <MA/gb300.hpp>

#include <cmath>
#include <cstdio>

struct Mat {
    std::vector<double> d;
    int64_t n = 0;
    int64_t rows() const { return n; }
    int64_t cols() const { return 2; }
    double operator()(int64_t i, int64_t j) const { return d[2 * i + j]; }
};

int main()
{
    const int W = 9, H = 7;  // image pixels: a W x H vertex grid of [-1, 1]^2
    try {
        MA::Density rho = MA::Density::image(std::vector<double>(W * H, 255.0), W, H);
        const double mass = rho.total_mass();
        Mat X;
        // generic coordinates: on the image's regular grid, round ones put bisectors
        // exactly through mesh vertices, and the drawing lists only cells whose pieces
        // need no exact predicate (MA_ERR_CAPACITY otherwise)
        X.d = {-0.4817, -0.3923, 0.2911, -0.1737, 0.6043, 0.6871, -0.2789, 0.5213, 0.1061, 0.0937};
        X.n = 5;
        const std::vector<double> w(5, 0.0), colors(5, 1.0);
        const size_t w_px = 16, h_px = 16;
        const double pixel_area = (2.0 / w_px) * (2.0 / h_px);
        const std::vector<double> img =
            MA::draw_laguerre_diagram(rho, X, w, colors, 1, -1.0, -1.0, 1.0, 1.0, w_px, h_px);
        double sum = 0.0;
        for (double v : img) sum += v;
        double sum_cb = 0.0;
        int calls = 0;
        MA::draw_laguerre_diagram(rho, X, w, colors, -1.0, -1.0, 1.0, 1.0, w_px, h_px, [&](int i, int j, double v) {
            if (i >= 0 && j >= 0 && i < (int)w_px && j < (int)h_px) sum_cb += v;
            calls++;
        });
        const double want = mass / pixel_area;
        std::printf("total mass %.15g, pixel sums %.15g / %.15g (want %.15g), %d put_pixel calls\n", mass, sum,
                    sum_cb, want, calls);
        if (std::fabs(mass - 4.0 * (1.0 + 1e-3)) > 1e-12 || std::fabs(sum - want) > 1e-9 * want ||
            std::fabs(sum_cb - sum) > 1e-12 * want || calls != (int)(w_px * h_px))
            return 4;
    } catch (const MA::Error& e) {
        std::printf("MA::Error: %s\n", e.what());
        return 3;
    }
    return 0;
}
