// Post-processing of a finished mesh on the device: area-weighted vertex
// normals (mesh_vertex_normals in include/meshing_gb300.h).
//
// One thread per face forms cross(v2 - v1, v3 - v1) in Float64 and adds it to
// its three vertices' accumulators (double atomics); one thread per vertex then
// normalizes.  The sums' order depends on scheduling, so normals agree with a
// sequential sum to rounding (about 1e-15 relative before the conversion to the
// vertex type), not bit for bit.
#include "mesh_host.h"
#include "mesh_internal.cuh"

#include <algorithm>

namespace mesh {
namespace {

template <class F>
__global__ void k_face_normals(const F *v, int64_t nv, const int64_t *f, int64_t nf, double *acc, unsigned *err) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id[3] = {f[3 * i] - 1, f[3 * i + 1] - 1, f[3 * i + 2] - 1};
        if (id[0] < 0 || id[0] >= nv || id[1] < 0 || id[1] >= nv || id[2] < 0 || id[2] >= nv) {
            atomicOr(err, ERR_BOUNDS);
            continue;
        }
        double p[3][3];
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) p[k][c] = (double)v[3 * id[k] + c];
        const double a[3] = {__dsub_rn(p[1][0], p[0][0]), __dsub_rn(p[1][1], p[0][1]), __dsub_rn(p[1][2], p[0][2])};
        const double b[3] = {__dsub_rn(p[2][0], p[0][0]), __dsub_rn(p[2][1], p[0][1]), __dsub_rn(p[2][2], p[0][2])};
        const double n[3] = {__dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1])),
                             __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2])),
                             __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]))};
#pragma unroll
        for (int k = 0; k < 3; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) atomicAdd(acc + 3 * id[k] + c, n[c]);
    }
}

template <class F> __global__ void k_normalize(const double *acc, int64_t nv, F *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = acc[3 * i], y = acc[3 * i + 1], z = acc[3 * i + 2];
        const double len = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z)));
        const double s = len > 0 ? __ddiv_rn(1.0, len) : 0.0;
        out[3 * i] = (F)__dmul_rn(x, s);
        out[3 * i + 1] = (F)__dmul_rn(y, s);
        out[3 * i + 2] = (F)__dmul_rn(z, s);
    }
}

template <class F>
cudaError_t normals_t(const void *verts, int64_t nv, const int64_t *faces, int64_t nf, void *out, double *acc,
                      unsigned *err, int sms, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(acc, 0, (size_t)nv * 3 * sizeof(double), s);
    if (e != cudaSuccess) return e;
    const int gf = (int)std::max<int64_t>(1, std::min<int64_t>((nf + 255) / 256, (int64_t)sms * 8));
    if (nf > 0) k_face_normals<F><<<gf, 256, 0, s>>>((const F *)verts, nv, faces, nf, acc, err);
    const int gv = (int)std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t)sms * 8));
    if (nv > 0) k_normalize<F><<<gv, 256, 0, s>>>(acc, nv, (F *)out);
    return cudaGetLastError();
}

}  // namespace
}  // namespace mesh

using namespace mesh;

extern "C" int mesh_vertex_normals(mesh_ctx *c, const void *verts, int float_bits, int64_t nverts,
                                   const int64_t *faces, int64_t nfaces, void *normals) {
    if (!c) return MESH_EINVAL;
    if ((float_bits != 32 && float_bits != 64) || nverts < 0 || nfaces < 0 ||
        (nverts > 0 && (!verts || !normals)) || (nfaces > 0 && !faces))
        return fail(c, MESH_EINVAL, "invalid normals arguments");
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    cudaError_t e;
    if ((e = c->misc.ensure(MISC_SLOTS * sizeof(int64_t))) != cudaSuccess) return cuda_fail(c, e, "misc buffer");
    if ((e = c->nrm.ensure((size_t)std::max<int64_t>(nverts, 1) * 3 * sizeof(double))) != cudaSuccess)
        return cuda_fail(c, e, "normal accumulators");
    // a fresh error word: mesh_ctx_sync reports what this call finds
    if ((e = cudaMemsetAsync(c->misc.ptr, 0, MISC_SLOTS * sizeof(int64_t), c->stream)) != cudaSuccess)
        return cuda_fail(c, e, "memset");
    unsigned *err = (unsigned *)((int64_t *)c->misc.ptr + NCNT);
    e = float_bits == 32 ? normals_t<float>(verts, nverts, faces, nfaces, normals, (double *)c->nrm.ptr, err, c->sms,
                                            c->stream)
                         : normals_t<double>(verts, nverts, faces, nfaces, normals, (double *)c->nrm.ptr, err, c->sms,
                                             c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "normals launch");
    c->have_plan = 0;  // the error word no longer belongs to an extraction
    return MESH_OK;
}
