// ma_raster.cu -- Laguerre-cell rasterisation into a device image.
//
// MA::draw_laguerre_diagram (include/MA/rasterization.hpp:516-547) walks every
// cell-triangle piece, takes the mean of the triangle's linear density at the piece's
// vertices, multiplies the cell's colour by it and rasterises the piece with exact
// pixel coverage (rasterize_convex_polygon, :403-480), handing cover x colour to a
// put_pixel callback.  Here the pieces come from the device listing (ma_pieces) and
// one warp per piece adds, for every pixel under the piece's box, the exact area of
// piece n pixel (Sutherland-Hodgman clip by the pixel's four sides, shoelace area)
// times the piece's colour into a headless image in device memory (FP64 atomics:
// the sums' last bits depend on the order of the pieces).  The reference nudges
// vertices off integer pixel coordinates by 1e-6 before its scanline pass; this
// computes the coverage of the unperturbed piece.
#include "ma_runtime.h"

namespace ma {

// the triangle's linear density at an absolute point
__device__ __forceinline__ double grid_rho(const MeshGridDev& m, int id, double x, double y)
{
    const int sq = id >> 1, i = sq % (m.nx - 1), j = sq / (m.nx - 1);
    const double* r0 = m.val + (size_t)j * m.nx;
    const double* r1 = r0 + m.nx;
    const double v00 = r0[i], v10 = r0[i + 1], v01 = r1[i], v11 = r1[i + 1];
    double gx, gy;
    if ((id & 1) == 0) {
        gx = (v10 - v00) * m.ihx[i];
        gy = (v11 - v10) * m.ihy[j];
    } else {
        gx = (v11 - v01) * m.ihx[i];
        gy = (v01 - v00) * m.ihy[j];
    }
    return v00 + gx * (x - m.gx[i]) + gy * (y - m.gy[j]);
}

__device__ __forceinline__ double tri_rho(const MeshTriDev& m, int t, double x, double y)
{
    const int a = m.tri[3 * t];
    return m.lin[3 * t] + m.lin[3 * t + 1] * (x - m.vx[a]) + m.lin[3 * t + 2] * (y - m.vy[a]);
}

constexpr int kRasterCap = 24;  // polygon vertices while a piece is clipped to a pixel

// area of polygon (px, py) (n vertices, counter-clockwise) inside [x0, x0+1] x [y0, y0+1];
// clipped and summed relative to the pixel's corner (terms of order 1)
__device__ __forceinline__ double pixel_cover(const double* px, const double* py, int n, double x0, double y0)
{
    double ax[kRasterCap], ay[kRasterCap], bx[kRasterCap], by[kRasterCap];
    int m = n;
    for (int k = 0; k < n; k++) {
        ax[k] = px[k] - x0;
        ay[k] = py[k] - y0;
    }
    // the four sides of [0, 1]^2: x >= 0, x <= 1, y >= 0, y <= 1, as  s * coord >= c
    for (int side = 0; side < 4 && m > 0; side++) {
        const bool isx = side < 2;
        const double sgn = (side & 1) ? -1.0 : 1.0;
        const double c = (side & 1) ? -1.0 : 0.0;
        int q = 0;
        for (int k = 0; k < m; k++) {
            const int k1 = k + 1 == m ? 0 : k + 1;
            const double d0 = sgn * (isx ? ax[k] : ay[k]) - c, d1 = sgn * (isx ? ax[k1] : ay[k1]) - c;
            if (d0 >= 0.0 && q < kRasterCap) {
                bx[q] = ax[k];
                by[q] = ay[k];
                q++;
            }
            if ((d0 >= 0.0) != (d1 >= 0.0) && q < kRasterCap) {
                const double t = d0 / (d0 - d1);
                bx[q] = ax[k] + t * (ax[k1] - ax[k]);
                by[q] = ay[k] + t * (ay[k1] - ay[k]);
                q++;
            }
        }
        m = q;
        for (int k = 0; k < m; k++) {
            ax[k] = bx[k];
            ay[k] = by[k];
        }
    }
    double a = 0.0;
    for (int k = 0; k < m; k++) {
        const int k1 = k + 1 == m ? 0 : k + 1;
        a += ax[k] * ay[k1] - ax[k1] * ay[k];
    }
    return 0.5 * a;
}

struct RasterArgs {
    int64_t npieces;
    const int* site;
    const int* tri;
    const int64_t* off;
    const double* xy;
    const double* colors;  // nc per site
    int nc;
    double x0, y0, sx, sy;  // image coordinates: (x - x0) sx, (y - y0) sy
    int w, h;
    double* image;          // h rows of w pixels of nc channels
};

template <class Rho>
__global__ void k_raster(RasterArgs a, Rho rho)
{
    const int64_t pc = (int64_t)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (pc >= a.npieces) return;
    const int64_t o0 = a.off[pc], o1 = a.off[pc + 1];
    const int n = (int)(o1 - o0);
    if (n < 3 || n > kRasterCap) return;
    double px[kRasterCap], py[kRasterCap];
    double ff = 0.0, bx0 = INFINITY, by0 = INFINITY, bx1 = -INFINITY, by1 = -INFINITY;
    const int t = a.tri[pc];
    for (int k = 0; k < n; k++) {
        const double x = a.xy[2 * (o0 + k)], y = a.xy[2 * (o0 + k) + 1];
        ff += rho(t, x, y);
        px[k] = (x - a.x0) * a.sx;
        py[k] = (y - a.y0) * a.sy;
        bx0 = fmin(bx0, px[k]);
        bx1 = fmax(bx1, px[k]);
        by0 = fmin(by0, py[k]);
        by1 = fmax(by1, py[k]);
    }
    ff /= n;  // the mean of the density at the piece's vertices (rasterization.hpp:530-536)
    const int i0 = max(0, (int)floor(bx0)), i1 = min(a.w - 1, (int)floor(bx1));
    const int j0 = max(0, (int)floor(by0)), j1 = min(a.h - 1, (int)floor(by1));
    if (i1 < i0 || j1 < j0) return;
    const int nw = i1 - i0 + 1;
    const int64_t npix = (int64_t)nw * (j1 - j0 + 1);
    const double* col = a.colors + (size_t)a.site[pc] * a.nc;
    for (int64_t q = lane; q < npix; q += 32) {
        const int i = i0 + (int)(q % nw), j = j0 + (int)(q / nw);
        const double cover = pixel_cover(px, py, n, (double)i, (double)j);
        if (!(cover > 0.0)) continue;
        double* pix = a.image + ((size_t)j * a.w + i) * a.nc;
        for (int c = 0; c < a.nc; c++) atomicAdd(&pix[c], cover * ff * col[c]);
    }
}

struct GridRho {
    MeshGridDev m;
    __device__ double operator()(int id, double x, double y) const { return grid_rho(m, id, x, y); }
};
struct TriRho {
    MeshTriDev m;
    __device__ double operator()(int id, double x, double y) const { return tri_rho(m, id, x, y); }
};

}  // namespace ma

using namespace ma;

extern "C" {

ma_status ma_draw_laguerre(ma_ctx* cp, const ma_mesh* mp, int64_t n, const double* x, const double* y,
                           const double* w, const double* colors, int channels, double x0, double y0, double x1,
                           double y1, int width, int height, double* image, ma_mem mem)
{
    Ctx* c = cp;
    const Mesh* m = mp;
    if (!c || !m || !colors || !image || channels < 1 || channels > 16 || width < 1 || height < 1 || !(x1 > x0) ||
        !(y1 > y0))
        return MA_ERR_INVALID_ARGUMENT;
    int64_t np = 0, nv = 0;
    ma_status st = ma_pieces(cp, mp, n, x, y, w, mem, &np, &nv);
    if (st != MA_OK) return st;
    cudaStream_t s = c->stream;
    const size_t npx = (size_t)width * height * channels;
    const double* dcol = colors;
    double* dimg = image;
    if (mem == MA_MEM_HOST) {
        MA_CUDA(c, c->raster_col.ensure(sizeof(double) * (size_t)n * channels));
        MA_CUDA(c, c->raster_img.ensure(sizeof(double) * npx));
        MA_CUDA(c, cudaMemcpyAsync(c->raster_col.p, colors, sizeof(double) * (size_t)n * channels,
                                   cudaMemcpyHostToDevice, s));
        MA_CUDA(c, cudaMemcpyAsync(c->raster_img.p, image, sizeof(double) * npx, cudaMemcpyHostToDevice, s));
        dcol = c->raster_col.as<double>();
        dimg = c->raster_img.as<double>();
    }
    RasterArgs a;
    a.npieces = np;
    a.site = c->pc_site.as<int>();
    a.tri = c->pc_tri.as<int>();
    a.off = c->pc_off.as<int64_t>();
    a.xy = c->pc_xy.as<double>();
    a.colors = dcol;
    a.nc = channels;
    a.x0 = x0;
    a.y0 = y0;
    a.sx = width / (x1 - x0);
    a.sy = height / (y1 - y0);
    a.w = width;
    a.h = height;
    a.image = dimg;
    if (np > 0) {
        const size_t threads = (size_t)np * 32;
        const unsigned g = (unsigned)((threads + 255) / 256);
        if (m->kind == 0)
            k_raster<<<g, 256, 0, s>>>(a, GridRho{m->grid_dev()});
        else
            k_raster<<<g, 256, 0, s>>>(a, TriRho{m->tri_dev()});
        c->launches += 1;
    }
    if (mem == MA_MEM_HOST)
        MA_CUDA(c, cudaMemcpyAsync(image, dimg, sizeof(double) * npx, cudaMemcpyDeviceToHost, s));
    MA_CUDA(c, cudaStreamSynchronize(s));
    return MA_OK;
}

}  // extern "C"
