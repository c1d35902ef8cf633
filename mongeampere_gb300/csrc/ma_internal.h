// ma_internal.h -- kernel launch interface shared by the host runtime and the
// kernels (not part of the public C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ma_cell.cuh"

namespace ma {

struct SiteGrid {
    int gnx, gny;
    double gx0, gy0, gcw, gch;  // cell (cx, cy) = [gx0 + cx gcw, ...) x [gy0 + cy gch, ...)
    const int* cell_start;      // gnx * gny + 1, positions in the sorted site array
};

// implicit grid mesh: vertex (i, j) at (gx[i], gy[j]) with value val[j * nx + i];
// square (i, j) is cut along its (i, j) -> (i+1, j+1) diagonal
struct MeshGridDev {
    int nx, ny;
    const double* gx;
    const double* gy;
    const double* val;
    const double* ihx;  // 1 / (gx[i+1] - gx[i])
    const double* ihy;
};

// explicit triangle mesh with a uniform bin index over its bounding box
struct MeshTriDev {
    int nv, nt;
    const double* vx;
    const double* vy;
    const int* tri;       // 3 per triangle, counter-clockwise
    const double* lin;    // 3 per triangle: rho(x) = lin0 + lin1 (x - v0.x) + lin2 (y - v0.y)
    const int4* tbin;     // per triangle: bin range bx0, by0, bx1, by1
    int bnx, bny;
    double bx0, by0, bcw, bch;
    const int* bin_start;  // bnx * bny + 1
    const int* bin_tri;
};

struct CellArgs {
    int n;
    const SiteD* sites;  // sorted by grid cell
    const int* perm;     // sorted position -> original index
    SiteGrid grid;
    double X0, Y0, X1, Y1;   // box of the cell stage (contains the mesh)
    const double* wmax;      // device scalar: max weight
    // outputs, original order
    double* mass;
    double* vpart;           // w_i m_i - int_{cell i} rho |x - x_i|^2
    double* mom;             // 6 per site or null: rho, rho x, rho y, rho x^2, rho y^2, rho x y
    int* rowcnt;
    int* st_col;
    double* st_val;
    int scap;
    uint32_t* status;
    int* redo;
    int* nredo;
    const int* work;         // when non-null, process only these sorted positions
    int nwork;
};

// launches (all asynchronous on `s`)
void launch_bbox(const double* x, const double* y, const double* w, int n, unsigned long long* keys,
                 cudaStream_t s);
void launch_grid_cells(const double* x, const double* y, int n, SiteGrid g, int* cell, int* count,
                       cudaStream_t s);
void launch_scatter(const int* cell, int n, const int* start, int* fill, int* perm, cudaStream_t s);
void launch_sort_cells(int ncell, const int* start, int* perm, cudaStream_t s);
void launch_gather(const double* x, const double* y, const double* w, const int* perm, int n, SiteD* out,
                   cudaStream_t s);
void launch_update_weights(const double* w, const int* perm, int n, SiteD* sites, cudaStream_t s);
void launch_wmax(const double* w, int n, unsigned long long* key, cudaStream_t s);
void launch_key_to_double(const unsigned long long* key, double* out, int count, cudaStream_t s);
void launch_scan(const int* in, int* out, int n, int* scratch, cudaStream_t s);  // exclusive, out has n+1
size_t scan_scratch_ints(int n);
void launch_cells_grid(const CellArgs& a, const MeshGridDev& m, int cap_kind, bool mom, cudaStream_t s);
void launch_cells_tri(const CellArgs& a, const MeshTriDev& m, int cap_kind, bool mom, cudaStream_t s);
void launch_csr_compact(int n, const int* rowptr, const int* rowcnt, const int* st_col, const double* st_val,
                        int scap, int* col, double* val, cudaStream_t s);

// deterministic reductions: out[0] = sum(vpart) - sum(nu * w) (if nu), [1] = sum(mass),
// [2] = min(mass), [3] = |mass - nu|_2, [4] = max |mass - nu| / nu
void launch_stats(const double* mass, const double* vpart, const double* nu, const double* w, int n,
                  double* partial, int nblocks, double* out, cudaStream_t s);
int stats_blocks(int n);

}  // namespace ma
