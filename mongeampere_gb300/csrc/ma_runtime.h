// ma_runtime.h -- host-side state behind the C ABI (context, meshes, buffers).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/ma.h"
#include "ma_internal.h"

namespace ma {

// grow-only device buffer
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need)
    {
        if (need <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t nb = need + need / 4 + 256;
        cudaError_t e = cudaMalloc(&p, nb);
        if (e == cudaSuccess) bytes = nb;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

struct Ctx;

struct Mesh {
    Ctx* ctx = nullptr;
    int kind = 0;  // 0 grid, 1 triangles
    double X0 = 0, Y0 = 0, X1 = 0, Y1 = 0;
    double total_mass = 0;
    // grid
    int nx = 0, ny = 0;
    DevBuf gx, gy, val, ihx, ihy;
    // triangles
    int nv = 0, nt = 0;
    DevBuf vx, vy, tri, lin, tbin, bin_start, bin_tri;
    int bnx = 0, bny = 0;
    double bx0 = 0, by0 = 0, bcw = 0, bch = 0;
    MeshGridDev grid_dev() const;
    MeshTriDev tri_dev() const;
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    std::string last_error;
    int64_t launches = 0;

    // inputs (when given in host memory)
    DevBuf hx, hy, hw, hnu;
    // site grid
    int n = 0;
    SiteGrid grid{};
    DevBuf cell, count, fill, start, perm, sites, scan_scratch;
    DevBuf keys, bboxd;  // ordered keys and their doubles
    // evaluation outputs
    DevBuf mass, vpart, mom, rowcnt, st_col, st_val, rowptr, col, val, status, redo, nredo, stat_partial, stat_out;
    DevBuf info;  // status, nredo, nnz
    int64_t nnz = 0;
    bool have_h = false;
    // solver work vectors
    DevBuf wcur, w0, dirn, g, cg_r, cg_z, cg_p, cg_q, cg_dinv, cg_scal, cg_part;
    // pinned host mirror of small results
    double* hstat = nullptr;  // 16 doubles
    int* hinfo = nullptr;     // 8 ints
};

// error helpers
ma_status fail(Ctx* c, ma_status s, const std::string& msg);
ma_status cuda_fail(Ctx* c, cudaError_t e, const char* what);

#define MA_CUDA(ctx, call)                                        \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return ::ma::cuda_fail(ctx, _e, #call); \
    } while (0)

// evaluation pipeline (device pointers)
ma_status build_site_grid(Ctx* c, const Mesh* m, int n, const double* x, const double* y, const double* w);
struct EvalFlags {
    bool hessian = true;
    int moments = 0;  // 0 none, 1 first, 2 second
    const double* nu = nullptr;  // when given, stat_out[0] = value - <nu, w>
};
ma_status run_eval(Ctx* c, const Mesh* m, int n, const double* w, const EvalFlags& f);

}  // namespace ma

// the opaque handles of the C ABI
struct ma_ctx : public ma::Ctx {};
struct ma_mesh : public ma::Mesh {};
