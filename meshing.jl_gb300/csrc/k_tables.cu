// Coordinate tables of the LinRange nodes, computed on the device.
//
// Replaces the node coordinates of mc_vert_points (src/marching_cubes.jl:111-120)
// and vertPos (src/marching_tetrahedra.jl:42-55): X, Y, Z become
// LinRange(first, last, n) whose i-th node is L((1 - t)*a + t*b), t = i/(n-1)
// (Base.lerpi), every operation rounded separately.  Layout (ntab = nx+ny+nz,
// nodes of x, then y, then z): node and spacing as double, the same as float,
// then the hi/lo float pairs of node and spacing used by the exact float path.
#include "mesh_internal.cuh"

#include <algorithm>

namespace mesh {

namespace {

// LinRange node coordinates, spacings and their float forms, computed on the
// device with the host path's arithmetic: L((1 - t)*a + t*b), t = i/(n-1), every
// operation rounded separately.
// Entry k of the table block at `tabs` for nx, ny, nz nodes.  The x nodes are
// nodes xoff .. xoff+nx-1 of an x axis of nxt nodes (a slab of a larger volume;
// xoff = 0, nxt = nx for a whole volume).
__device__ __forceinline__ void table_entry(double *tabs, int64_t k, int64_t nx, int64_t ny, int64_t nz, double x0,
                                            double x1, double y0, double y1, double z0, double z1, int L32,
                                            int64_t xoff = 0, int64_t nxt = 0) {
    const int64_t ntab = nx + ny + nz;
    double *hp = tabs, *hd = tabs + ntab;
    float *hpf = (float *)(tabs + 2 * ntab), *hdf = hpf + ntab, *hs = hdf + ntab;
    int64_t i = k + xoff, n = nxt > 0 ? nxt : nx;
    double a = x0, b = x1;
    if (k >= nx + ny) {
        i = k - nx - ny; n = nz; a = z0; b = z1;
    } else if (k >= nx) {
        i = k - nx; n = ny; a = y0; b = y1;
    }
    if (L32) {
        a = (double)(float)a;
        b = (double)(float)b;
    }
    const double dn = (double)(n > 1 ? n - 1 : 1);
    auto node = [&](int64_t j) {
        const double t = __ddiv_rn((double)j, dn);
        const double v = __dadd_rn(__dmul_rn(__dsub_rn(1.0, t), a), __dmul_rn(t, b));
        return L32 ? (double)(float)v : v;
    };
    const double v = node(i);
    double d = 0;
    if (i + 1 < n) {
        const double v1 = node(i + 1);
        d = L32 ? (double)__fsub_rn((float)v1, (float)v) : __dsub_rn(v1, v);
    }
    hp[k] = v;
    hd[k] = d;
    hpf[k] = (float)v;
    hdf[k] = (float)d;
    hs[k] = (float)v;
    hs[ntab + k] = (float)__dsub_rn(v, (double)(float)v);
    hs[2 * ntab + k] = (float)d;
    hs[3 * ntab + k] = (float)__dsub_rn(d, (double)(float)d);
}

__global__ void k_tables(double *tabs, int64_t nx, int64_t ny, int64_t nz, double x0, double x1, double y0,
                         double y1, double z0, double z1, int L32, int64_t xoff, int64_t nxt) {
    const int64_t ntab = nx + ny + nz;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ntab; k += (int64_t)gridDim.x * blockDim.x)
        table_entry(tabs, k, nx, ny, nz, x0, x1, y0, y1, z0, z1, L32, xoff, nxt);
}

__global__ void k_tables_batch(const TabJob *jobs, int L32) {
    const TabJob &j = jobs[blockIdx.y];
    const int64_t ntab = j.nx + j.ny + j.nz;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ntab; k += (int64_t)gridDim.x * blockDim.x)
        table_entry(j.dst, k, j.nx, j.ny, j.nz, j.range[0], j.range[1], j.range[2], j.range[3], j.range[4],
                    j.range[5], L32);
}

}  // namespace

cudaError_t launch_tables_batch(const TabJob *jobs, int njobs, int64_t max_ntab, int L32, cudaStream_t s) {
    for (int j0 = 0; j0 < njobs; j0 += 65535) {  // grid y limit
        const int nj = std::min(65535, njobs - j0);
        dim3 grid((unsigned)std::min<int64_t>((max_ntab + 255) / 256, 64), (unsigned)nj);
        k_tables_batch<<<grid, 256, 0, s>>>(jobs + j0, L32);
    }
    return cudaGetLastError();
}

cudaError_t launch_tables(double *tabs, int64_t nx, int64_t ny, int64_t nz, const double *range, int L32,
                          cudaStream_t s, int64_t xoff, int64_t nxt) {
    const int64_t ntab = nx + ny + nz;
    k_tables<<<(int)std::min<int64_t>((ntab + 255) / 256, 1024), 256, 0, s>>>(
        tabs, nx, ny, nz, range[0], range[1], range[2], range[3], range[4], range[5], L32, xoff, nxt);
    return cudaGetLastError();
}

}  // namespace mesh
