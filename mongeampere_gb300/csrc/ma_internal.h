// ma_internal.h -- kernel launch interface shared by the host runtime and the
// kernels (not part of the public C ABI).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ma_cell.cuh"

namespace ma {

// binary radix tree over the Morton-sorted sites; internal node 0 is the root;
// a child index with the top bit set is a leaf (sorted site position)
struct SiteTree {
    int n;
    const int2* child;
    const int2* range;    // first, last sorted position covered by the node
    const double4* box;   // x0, y0, x1, y1 (exact)
    const float4* boxf;   // the same rounded outwards
    const double4* ab;    // alpha, beta_x, beta_y: phi_j >= alpha + beta . x_j over the node
    const float4* nk;     // the same about the FP32 box centre c: A = alpha + beta.c - |c|^2/2
                          // (rounded down), beta_x - c_x, beta_y - c_y, 0
    const float2* posf;   // sorted site positions (FP32)
    const int* parent;      // parent of each internal node (-1 at the root)
    const int* leaf_parent; // parent of each leaf
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
    SiteTree tree;
    double X0, Y0, X1, Y1;   // box of the cell stage (contains the mesh)
    // outputs, original order
    double* mass;
    double* vpart;           // w_i m_i - int_{cell i} rho |x - x_i|^2
    int value = 1;           // 0: the grid-piece integrals leave out int rho |x - x_i|^2
                             // (vpart then holds w_i m_i only)
    double* mom;             // 6 per site or null: rho, rho x, rho y, rho x^2, rho y^2, rho x y
    int* rowcnt;
    int* st_col;
    double* st_val;
    int scap;
    uint32_t* status;
    int* redo;
    int* nredo;
    const int* work;         // large-capacity pass: the sorted positions to redo
    int nwork;
    int prev_valid;          // nb_cnt / nb_lab hold the previous evaluation's lists for these sites
    int* nb_cnt;             // stage 1 -> 2, sorted order: neighbour count, -1 empty cell, -2 large pass
    int* nb_lab;             // stage 1 -> 2: neighbour sorted indices, stage1_cap() per site
    double4* cell_box;       // stage 1 -> 2: absolute bounding box of the cell
    unsigned long long* counters;  // optional stage-1 search counters (6)
    int* abort_flag;         // optional: set at the first empty cell, and every cell then stops
    // adjoint (k_pieces in its VJP mode): cotangents of the value, the masses and
    // the first moments int rho x (2 per site), and the gradients (original order;
    // grad_rho per mesh vertex, accumulated with atomics)
    double cot_value;
    const double* cot_mass;
    const double* cot_mom;
    double* grad_x;
    double* grad_y;
    double* grad_w;
    double* grad_rho;
    // materialised pieces (k_pieces in its count and emit modes), cells in sorted order
    int* pc_cnt;         // count: pieces per cell
    int* pv_cnt;         // count: polygon vertices per cell
    const int* pc_base;  // emit: first piece of each cell
    const int* pv_base;  // emit: first vertex of each cell
    int* out_site;       // emit, per piece: site (original index)
    int* out_tri;        //                  mesh triangle
    int64_t* out_off;    //                  first vertex
    double* out_xy;      // emit, per vertex: absolute position (x, y)
    int* out_edge;       //                  the edge starting there: neighbour site, or -1-e for triangle edge e
    const int* cell_list;    // k_pieces: the sorted indices of the cells to do (null: all n)
    int ncell_list;
    int* redo64;             // mixed form: cells whose certified FP32 mass error is too large,
    int* nredo64;            // redone by the FP64 pieces kernel
    void* scratch;           // large-capacity pass: one workspace per work item
    int* big_index;          // per site: row slot in the side buffer, -1 otherwise
    int* big_col;
    double* big_val;
    int big_cap;
};

// launches (all asynchronous on `s`)
void launch_bbox(const double* x, const double* y, const double* w, int n, unsigned long long* keys,
                 cudaStream_t s);
void launch_update_weights(const double* w, const int* perm, int n, SiteD* sites, cudaStream_t s);
void launch_key_to_double(const unsigned long long* key, double* out, int count, cudaStream_t s);
// site index (ma_index.cu)
void launch_morton(const double* x, const double* y, int n, double x0, double y0, double x1, double y1,
                   uint64_t* keys, cudaStream_t s);
int radix_sort_blocks(int n);
void launch_radix_sort(uint64_t* keys, uint64_t* tmp, int n, int* hist, int* hist_scan, int* scan_scratch,
                       cudaStream_t s);
void launch_perm_gather(const uint64_t* keys, const double* x, const double* y, const double* w, int n, int* perm,
                        SiteD* sites, float2* posf, cudaStream_t s);
void launch_tree(const uint64_t* keys, int n, int2* child, int2* range, int* parent, int* leaf_parent,
                 cudaStream_t s);
void launch_tree_boxes(const SiteD* sites, int n, const int2* child, const int* parent, const int* leaf_parent,
                       int* flag, double4* box, float4* boxf, cudaStream_t s);
size_t tree_mom_bytes(int n);
inline int tree_bounds_launches(int n) { return n < 2 ? 0 : 3; }
void launch_tree_bounds(const SiteD* sites, int n, const int2* child, const int2* range, const int* parent,
                        const int* leaf_parent, int* flag, const double4* box, const float4* boxf, void* mom,
                        double4* ab, float4* nk, cudaStream_t s);
void launch_scan(const int* in, int* out, int n, int* scratch, cudaStream_t s);  // exclusive, out has n+1
size_t scan_scratch_ints(int n);
// cell kernels (ma_cells.cu)
void launch_cells_stage1(const CellArgs& a, cudaStream_t s);
// mode: 0 evaluation, 1 evaluation with moments, 2 adjoint (vector-Jacobian product),
// 3 count the pieces per cell, 4 emit them, 5 evaluation with FP32 piece integrals, 6 the
// adjoint with FP32 piece integrals
void launch_pieces_grid(const CellArgs& a, const MeshGridDev& m, int mode, cudaStream_t s);
void launch_pieces_tri(const CellArgs& a, const MeshTriDev& m, int mode, cudaStream_t s);
void launch_cells_large_grid(const CellArgs& a, const MeshGridDev& m, bool mom, cudaStream_t s);
void launch_cells_large_tri(const CellArgs& a, const MeshTriDev& m, bool mom, cudaStream_t s);
int stage1_cap();
// the pieces of the cells a.work[0..a.nwork) (sorted indices), one thread per cell with
// exact predicates: count them (pc_cnt, pv_cnt; the cells' nb_cnt become -3 so that the
// warp kernel's emit pass leaves them) or emit them; a cell beyond every capacity adds 1
// to *a.nredo.  g (grid) or tm (triangles) is the mesh.
void launch_cells_large_list(const CellArgs& a, const MeshGridDev* g, const MeshTriDev* tm, bool emit,
                             cudaStream_t s);
void launch_csr_compact(int n, const int* rowptr, const int* rowcnt, const int* st_col, const double* st_val,
                        int scap, const int* big_index, const int* big_col, const double* big_val, int big_cap,
                        int* col, double* val, cudaStream_t s);
size_t large_work_bytes();
int large_row_cap();
int small_row_cap();

// deterministic reductions: out[0] = sum(vpart) - sum(nu * w) (if nu), [1] = sum(mass),
// [2] = min(mass), [3] = |mass - nu|_2, [4] = max |mass - nu| / nu
void launch_stats(const double* mass, const double* vpart, const double* nu, const double* w, int n,
                  double* partial, int nblocks, double* out, cudaStream_t s);
int stats_blocks(int n);

}  // namespace ma
