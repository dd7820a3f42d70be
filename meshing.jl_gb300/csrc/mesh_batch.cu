// Batched Marching Cubes behind the C ABI (mesh_batch_* in include/meshing_gb300.h).
//
// Many volumes of uneven shape are extracted by one pass of each stage over a
// flattened worklist instead of one launch sequence per volume:
//   classify  persistent warps over all volumes' warp tiles (k_classify_batch)
//   scan      one decoupled look-back chain over all volumes' scan tiles, so
//             the volumes' meshes are concatenated in volume order, plus the
//             first vertex / face of every volume (k_scan_batch)
//   compact   persistent warps list the active cells (k_compact_batch)
//   expand    vertices and faces, faces 1-based within their volume
// Each volume gives the same vertices and faces, in the same order, as a call
// of isosurface(A_i, MarchingCubes(iso), X_i, Y_i, Z_i) on it alone
// (src/marching_cubes.jl:27-64).
//
// The run after a count can be captured once into a CUDA graph and replayed.
// The autotuner times the whole sequence over a small set of brick depths
// (z cells per work item), persistent CTAs per SM and scan CTA widths, one
// knob at a time, and keeps the fastest.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mesh_host.h"
#include "mesh_internal.cuh"

using namespace mesh;

struct mesh_batch {
    mesh_ctx *ctx = nullptr;
    int n = 0, T = 0;
    mesh_params prm{};
    int Q64 = 0, A64 = 0, P64 = 0;
    std::vector<const void *> vols;
    std::vector<int64_t> dims;    // [n][3]
    std::vector<double> ranges;   // [n][6]
    // tunables
    int zs = 0;                   // z cells per work item, a multiple of ZC; 0 = whole columns
    int cls_ctas = 0, cmp_ctas = 0;  // CTAs per SM of the persistent kernels; 0 = as many as fit
    int scan_threads = 1024;
    bool scan_vol = false;        // every volume at most 4 column groups wide: the per-volume scan
    Plan P{};
    std::vector<BatchVol> hv;
    DevBuf dvols, ivol, svol, tabs, jobs, cnt, base, flags, scan, misc, ent, out_v, out_f, offs;
    int64_t *h_misc = nullptr;    // pinned copy of the misc words
    int64_t nverts = 0, nfaces = 0, nactive = 0;
    int counted = 0;
    int use_graph = 0;
    // welded batches: the per-cell mesh goes to out_v / out_f, its edge keys to
    // wkey; the welded vertices to wv, the faces are renumbered in place, the
    // welded rows to woffs
    int weld = 0;
    int64_t nv_cell = 0;          // per-cell vertices at the last count
    DevBuf wkey, wbuf, wv, woffs;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t cap = nullptr;   // capture stream (the legacy default stream cannot be captured)
};

namespace mesh {

BatchSizes tile_batch(const int64_t *dims, int n, int zs, std::vector<BatchVol> &hv, std::vector<int64_t> &tab_off) {
    BatchSizes z;
    hv.assign(n, BatchVol{});
    tab_off.assign(n, 0);
    for (int v = 0; v < n; v++) {
        BatchVol &bv = hv[v];
        const int64_t nx = dims[3 * v], ny = dims[3 * v + 1], nz = dims[3 * v + 2];
        bv.nx = nx; bv.ny = ny; bv.nz = nz;
        bv.item0 = z.items; bv.piece0 = z.pieces; bv.flag0 = z.nflags; bv.stile0 = (int32_t)z.stiles;
        bv.kbase = z.keys;
        z.keys += 3 * nx * ny * nz;
        tab_off[v] = z.tdoubles;
        if (nx < 2 || ny < 2 || nz < 2) {  // no cells: an empty mesh
            bv.zs = ZC; bv.chunks_per_seg = 1;
            continue;
        }
        bv.cx = (int32_t)(nx - 1); bv.cy = (int32_t)(ny - 1); bv.cz = (int32_t)(nz - 1);
        bv.tiles_x = (bv.cx + TILE_X - 1) / TILE_X;
        bv.tiles_y = (bv.cy + WY - 1) / WY;
        const int whole = (bv.cz + ZC - 1) / ZC * ZC;
        bv.zs = zs > 0 ? std::min(whole, (zs + ZC - 1) / ZC * ZC) : whole;
        bv.nseg = (bv.cz + bv.zs - 1) / bv.zs;
        bv.chunks_per_seg = bv.zs / ZC;
        bv.nchunks = bv.nseg * bv.chunks_per_seg;
        z.items += (int64_t)bv.tiles_x * bv.tiles_y * bv.nseg;
        z.pieces += (int64_t)bv.nseg * bv.cy * bv.cx;
        z.nflags += (int64_t)bv.nchunks * bv.tiles_x * bv.cy;
        z.stiles += (bv.cx + 31) / 32;
        const int64_t ntab = nx + ny + nz;
        z.max_ntab = std::max(z.max_ntab, ntab);
        z.tdoubles += (int64_t)((table_bytes(ntab) + 255) / 256 * 32);  // 256-byte aligned blocks
    }
    return z;
}

void batch_owners(const std::vector<BatchVol> &hv, const BatchSizes &z, std::vector<uint32_t> &ivol,
                  std::vector<uint32_t> &svol) {
    ivol.resize((size_t)z.items);
    svol.resize((size_t)z.stiles);
    for (size_t v = 0; v < hv.size(); v++) {
        const BatchVol &bv = hv[v];
        if (!bv.cx) continue;
        const int64_t ni = (int64_t)bv.tiles_x * bv.tiles_y * bv.nseg;
        std::fill(ivol.begin() + bv.item0, ivol.begin() + bv.item0 + ni, (uint32_t)v);
        const int ns = (bv.cx + 31) / 32;
        std::fill(svol.begin() + bv.stile0, svol.begin() + bv.stile0 + ns, (uint32_t)v);
    }
}

}  // namespace mesh

namespace {

void drop_graph(mesh_batch *b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
}

// Work items, pieces, activity bytes, scan tiles and tables of every volume.
int build_plan(mesh_batch *b) {
    mesh_ctx *c = b->ctx;
    drop_graph(b);
    b->counted = 0;
    Plan &P = b->P;
    P = Plan{};
    set_types(P, b->T, &b->prm, &b->Q64, &b->A64, &b->P64);
    const int L32 = b->prm.range_type == MESH_DT_F32;
    const int n = b->n;
    std::vector<int64_t> tab_off;
    const BatchSizes z = tile_batch(b->dims.data(), n, b->zs, b->hv, tab_off);
    for (int v = 0; v < n; v++) b->hv[v].vol = b->vols[v];
    const int64_t items = z.items, pieces = z.pieces, nflags = z.nflags, tdoubles = z.tdoubles, stiles = z.stiles;
    const int64_t max_ntab = z.max_ntab;
    // the compaction splits each item into up to WY row tiles counted in 32 bits
    if (items >= ((int64_t)1 << 31) / WY || stiles >= ((int64_t)1 << 31))
        return fail(c, MESH_ETOOLARGE, "batch has too many work items");

    cudaError_t e;
    const size_t bvb = sizeof(BatchVol) * (size_t)std::max(n, 1);
    if ((e = b->dvols.ensure(bvb)) != cudaSuccess || (e = b->ivol.ensure(4 * (size_t)items + 4)) != cudaSuccess ||
        (e = b->svol.ensure(4 * (size_t)stiles + 4)) != cudaSuccess ||
        (e = b->tabs.ensure(8 * (size_t)tdoubles + 8)) != cudaSuccess ||
        (e = b->jobs.ensure(sizeof(TabJob) * (size_t)std::max(n, 1))) != cudaSuccess ||
        (e = b->cnt.ensure((size_t)pieces * NCNT * 4 + 4)) != cudaSuccess ||
        (e = b->base.ensure((size_t)pieces * NCNT * 8 + 8)) != cudaSuccess ||
        (e = b->flags.ensure((size_t)nflags + 1)) != cudaSuccess ||
        (e = b->scan.ensure((size_t)std::max<int64_t>(stiles, n) * NCNT * 8 + 64)) != cudaSuccess ||
        (e = b->misc.ensure(MISC_SLOTS * sizeof(int64_t))) != cudaSuccess ||
        (e = b->offs.ensure((size_t)(n + 1) * 2 * 8)) != cudaSuccess)
        return cuda_fail(c, e, "batch buffers");

    // per-volume tables, item and scan-tile owners
    std::vector<TabJob> jobs;
    std::vector<uint32_t> ivol, svol;
    batch_owners(b->hv, z, ivol, svol);
    for (int v = 0; v < n; v++) {
        BatchVol &bv = b->hv[v];
        bv.tabs = (const double *)b->tabs.ptr + tab_off[v];
        if (!bv.cx) continue;
        TabJob j;
        j.dst = (double *)b->tabs.ptr + tab_off[v];
        j.nx = bv.nx; j.ny = bv.ny; j.nz = bv.nz;
        for (int k = 0; k < 6; k++) j.range[k] = b->ranges[6 * v + k];
        jobs.push_back(j);
    }
    // plan building is off the hot path: plain synchronous uploads
    if ((e = cudaMemcpy(b->dvols.ptr, b->hv.data(), sizeof(BatchVol) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (items && (e = cudaMemcpy(b->ivol.ptr, ivol.data(), 4 * (size_t)items, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (stiles && (e = cudaMemcpy(b->svol.ptr, svol.data(), 4 * (size_t)stiles, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (!jobs.empty() &&
         (e = cudaMemcpy(b->jobs.ptr, jobs.data(), sizeof(TabJob) * jobs.size(), cudaMemcpyHostToDevice)) != cudaSuccess))
        return cuda_fail(c, e, "batch plan upload");
    if (!jobs.empty() && (e = launch_tables_batch((const TabJob *)b->jobs.ptr, (int)jobs.size(), max_ntab, L32,
                                                  c->stream)) != cudaSuccess)
        return cuda_fail(c, e, "batch tables");

    P.force_fp64 = c->force_fp64;
    P.pstride = pieces;
    P.cnt = (uint32_t *)b->cnt.ptr;
    P.base = (int64_t *)b->base.ptr;
    P.flags = (uint8_t *)b->flags.ptr;
    P.scan_state = (unsigned long long *)b->scan.ptr;
    P.scan_ticket = (unsigned int *)((char *)b->scan.ptr + (size_t)std::max<int64_t>(stiles, n) * NCNT * 8);
    b->scan_vol = true;
    for (const BatchVol &bv : b->hv) b->scan_vol = b->scan_vol && bv.cx <= 4 * 32;
    P.totals = (int64_t *)b->misc.ptr;
    P.err = (unsigned int *)((int64_t *)b->misc.ptr + NCNT);
    P.work = (unsigned int *)((int64_t *)b->misc.ptr + NCNT + 1);
    P.scan_spin_limit = 1 << 24;
    P.bvols = (const BatchVol *)b->dvols.ptr;
    P.item_vol = (const uint32_t *)b->ivol.ptr;
    P.stile_vol = (const uint32_t *)b->svol.ptr;
    P.vol_off = (int64_t *)b->offs.ptr;
    P.nitems = items;
    P.nvols = n;
    P.nstiles = (int32_t)stiles;
    return MESH_OK;
}

int fetch(mesh_batch *b) {
    mesh_ctx *c = b->ctx;
    cudaError_t e = cudaMemcpyAsync(b->h_misc, b->misc.ptr, MISC_SLOTS * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "batch synchronize");
    const unsigned err = (unsigned)(b->h_misc[NCNT] & 0xffffffffll);
    if (err & ERR_SCAN_TIMEOUT) return fail(c, MESH_EDEVICE, "scan look-back wait expired");
    if (err & ERR_BOUNDS) return fail(c, MESH_EDEVICE, "device bounds check failed");
    if (err & ERR_CAPACITY) return fail(c, MESH_ECAPACITY, "batch outputs larger than at the last count");
    return MESH_OK;
}

// classify + scan (with the per-volume offsets), on stream s
int enqueue_count(mesh_batch *b, cudaStream_t s) {
    mesh_ctx *c = b->ctx;
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->misc.ptr, 0, MISC_SLOTS * sizeof(int64_t), s)) != cudaSuccess)
        return cuda_fail(c, e, "memset");
    if ((e = launch_classify_batch(b->P, b->cls_ctas, s)) != cudaSuccess) return cuda_fail(c, e, "batch classify");
    if ((e = launch_scan_batch(b->P, b->scan_threads, s, b->scan_vol)) != cudaSuccess)
        return cuda_fail(c, e, "batch scan");
    return MESH_OK;
}

int enqueue_run(mesh_batch *b, cudaStream_t s) {
    int rc = enqueue_count(b, s);
    if (rc) return rc;
    mesh_ctx *c = b->ctx;
    cudaError_t e;
    if ((e = launch_compact_batch(b->P, b->cmp_ctas, s)) != cudaSuccess) return cuda_fail(c, e, "batch compact");
    if ((e = launch_expand_batch(b->P, b->Q64, b->P64, s)) != cudaSuccess) return cuda_fail(c, e, "batch expand");
    if (b->weld) {
        const Plan &P = b->P;
        const int64_t nb = weld_blocks(b->nv_cell), hcap = weld_hash_slots(b->nv_cell);
        char *wb = (char *)b->wbuf.ptr;
        const size_t o_hkey = ((size_t)(nb + 1) * 8 + 255) / 256 * 256, o_hval = o_hkey + (size_t)hcap * 8;
        if ((e = launch_weld_batch(P.vkey, b->nv_cell, b->nfaces, P.totals, P.verts, P.out64, P.faces, P.vol_off, b->n,
                                   (int64_t *)b->woffs.ptr, (long long *)wb, b->wv.ptr,
                                   (unsigned long long *)(wb + o_hkey), (long long *)(wb + o_hval), hcap, P.err,
                                   c->sms, s)) != cudaSuccess)
            return cuda_fail(c, e, "batch weld");
    }
    return MESH_OK;
}

int count(mesh_batch *b) {
    mesh_ctx *c = b->ctx;
    drop_graph(b);
    int rc = enqueue_count(b, c->stream);
    if (rc || (rc = fetch(b))) return rc;
    b->nverts = b->h_misc[0];
    b->nfaces = b->h_misc[1];
    b->nactive = b->h_misc[2];
    Plan &P = b->P;
    // active-cell list (emission order over the batch) and the outputs, sized exactly
    const size_t es = dtype_size(b->T);
    const int64_t cap = b->nactive;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t o_val = up((size_t)cap * 8);
    const size_t o_side = o_val + up((size_t)cap * 8 * es);
    const size_t o_vol = o_side + up((size_t)(cap / ENT_BLOCK + 1) * 16);
    const size_t o_cs = o_vol + up((size_t)cap * 4);
    const size_t vb = (size_t)b->nverts * 3 * (P.out64 ? 8 : 4), fb = (size_t)b->nfaces * 3 * 8;
    cudaError_t e;
    if ((e = b->ent.ensure(o_cs + up((size_t)cap + 1))) != cudaSuccess || (e = b->out_v.ensure(vb + 16)) != cudaSuccess ||
        (e = b->out_f.ensure(fb + 16)) != cudaSuccess)
        return cuda_fail(c, e, "batch outputs");
    char *eb = (char *)b->ent.ptr;
    P.ent_pos = (unsigned long long *)eb;
    P.ent_val = eb + o_val;
    P.ent_side = (long long *)(eb + o_side);
    P.ent_vol = (uint32_t *)(eb + o_vol);
    P.ent_cs = (uint8_t *)(eb + o_cs);
    P.ent_cap = cap;
    P.verts = b->out_v.ptr;
    P.faces = (int64_t *)b->out_f.ptr;
    P.verts_cap = b->nverts;
    P.faces_cap = b->nfaces;
    P.vkey = nullptr;
    b->counted = 1;
    if (!b->weld) return MESH_OK;
    // welded: edge keys, weld scratch, welded vertices and rows; one whole run
    // (per-cell mesh and weld) sizes the welded vertices exactly
    b->nv_cell = b->nverts;
    const int64_t nb = weld_blocks(b->nv_cell), hcap = weld_hash_slots(b->nv_cell);
    const size_t wbytes = up((size_t)(nb + 1) * 8) + (size_t)hcap * 16;
    if ((e = b->wkey.ensure((size_t)b->nv_cell * 8 + 16)) != cudaSuccess || (e = b->wbuf.ensure(wbytes)) != cudaSuccess ||
        (e = b->wv.ensure(vb + 16)) != cudaSuccess || (e = b->woffs.ensure((size_t)(b->n + 1) * 16)) != cudaSuccess)
        return cuda_fail(c, e, "weld buffers");
    P.vkey = (long long *)b->wkey.ptr;
    if ((rc = enqueue_run(b, c->stream)) || (rc = fetch(b))) return rc;
    int64_t row[2];
    if ((e = cudaMemcpy(row, (int64_t *)b->woffs.ptr + 2 * (size_t)b->n, sizeof(row), cudaMemcpyDeviceToHost)) !=
        cudaSuccess)
        return cuda_fail(c, e, "welded totals");
    b->nverts = row[0];
    return MESH_OK;
}

int run(mesh_batch *b) {
    mesh_ctx *c = b->ctx;
    if (!b->counted) return fail(c, MESH_ESTATE, "mesh_batch_run without mesh_batch_count");
    cudaError_t e;
    if (!b->use_graph) return enqueue_run(b, c->stream);
    if (!b->gexec) {
        // captured on a private stream, launched on the context's
        if (!b->cap && (e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess)
            return cuda_fail(c, e, "capture stream");
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed)) != cudaSuccess)
            return cuda_fail(c, e, "graph capture");
        const int rc = enqueue_run(b, b->cap);
        e = cudaStreamEndCapture(b->cap, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(c, e, "graph capture");
        e = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->gexec = nullptr;
            return cuda_fail(c, e, "graph instantiate");
        }
    }
    if ((e = cudaGraphLaunch(b->gexec, c->stream)) != cudaSuccess) return cuda_fail(c, e, "graph launch");
    return MESH_OK;
}

// Median device time of `reps` runs, in ms.
int time_runs(mesh_batch *b, int reps, double *ms) {
    mesh_ctx *c = b->ctx;
    std::vector<cudaEvent_t> ev(2 * reps);
    for (auto &x : ev) cudaEventCreate(&x);
    int rc = run(b);  // warm-up (and graph instantiation)
    for (int i = 0; !rc && i < reps; i++) {
        cudaEventRecord(ev[2 * i], c->stream);
        rc = run(b);
        cudaEventRecord(ev[2 * i + 1], c->stream);
    }
    if (!rc) rc = fetch(b);
    std::vector<double> t;
    for (int i = 0; !rc && i < reps; i++) {
        float x = 0;
        cudaEventElapsedTime(&x, ev[2 * i], ev[2 * i + 1]);
        t.push_back(x);
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    std::sort(t.begin(), t.end());
    *ms = t[t.size() / 2];
    return MESH_OK;
}

}  // namespace

extern "C" {

int mesh_batch_create(mesh_ctx *ctx, int n, const void *const *vols, int dtype, const int64_t *dims,
                      const mesh_params *p, const double *ranges, mesh_batch **out) {
    if (!ctx || !out || n < 0 || (n > 0 && (!vols || !dims))) return fail(ctx, MESH_EINVAL, "NULL argument");
    *out = nullptr;
    ctx->msg.clear();
    if (!p) return fail(ctx, MESH_EINVAL, "params is NULL");
    if (p->alg != MESH_ALG_MC && p->alg != MESH_ALG_MC_WELDED)
        return fail(ctx, MESH_EINVAL, "batches run MarchingCubes only");
    for (int v = 0; v < n; v++) {
        mesh_params q = *p;
        if (ranges) memcpy(q.range, ranges + 6 * v, sizeof(q.range));
        int rc = validate(ctx, dtype, dims[3 * v], dims[3 * v + 1], dims[3 * v + 2], &q);
        if (rc) return rc;
        const bool cells = dims[3 * v] > 1 && dims[3 * v + 1] > 1 && dims[3 * v + 2] > 1;
        if (cells && !vols[v]) return fail(ctx, MESH_EINVAL, "volume %d is NULL", v);
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, MESH_ECUDA, "cudaSetDevice");
    mesh_batch *b = new (std::nothrow) mesh_batch();
    if (!b) return fail(ctx, MESH_ENOMEM, "batch");
    b->ctx = ctx;
    b->n = n;
    b->T = dtype;
    b->prm = *p;
    b->weld = p->alg == MESH_ALG_MC_WELDED;
    b->prm.alg = MESH_ALG_MC;  // welded batches run the Marching Cubes kernels, then weld
    b->vols.assign(vols, vols + n);
    b->dims.assign(dims, dims + 3 * n);
    b->ranges.resize(6 * (size_t)n);
    for (int v = 0; v < n; v++)
        for (int k = 0; k < 6; k++) b->ranges[6 * v + k] = ranges ? ranges[6 * v + k] : p->range[k];
    if (cudaHostAlloc((void **)&b->h_misc, MISC_SLOTS * sizeof(int64_t), cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return fail(ctx, MESH_ENOMEM, "pinned batch words");
    }
    int rc = build_plan(b);
    if (rc) {
        mesh_batch_destroy(b);
        return rc;
    }
    *out = b;
    return MESH_OK;
}

void mesh_batch_destroy(mesh_batch *b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    drop_graph(b);
    DevBuf *bufs[] = {&b->dvols, &b->ivol, &b->svol,  &b->tabs, &b->jobs, &b->cnt,  &b->base, &b->flags, &b->scan,
                      &b->misc,  &b->ent,  &b->out_v, &b->out_f, &b->offs, &b->wkey, &b->wbuf, &b->wv,   &b->woffs};
    for (DevBuf *x : bufs) x->release();
    if (b->h_misc) cudaFreeHost(b->h_misc);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
}

int mesh_batch_count(mesh_batch *b, int64_t *nverts, int64_t *nfaces) {
    if (!b || !nverts || !nfaces) return MESH_EINVAL;
    b->ctx->msg.clear();
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return fail(b->ctx, MESH_ECUDA, "cudaSetDevice");
    int rc = count(b);
    if (rc) return rc;
    *nverts = b->nverts;
    *nfaces = b->nfaces;
    return MESH_OK;
}

int mesh_batch_run(mesh_batch *b) {
    if (!b) return MESH_EINVAL;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return fail(b->ctx, MESH_ECUDA, "cudaSetDevice");
    return run(b);
}

int mesh_batch_sync(mesh_batch *b) {
    if (!b) return MESH_EINVAL;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return fail(b->ctx, MESH_ECUDA, "cudaSetDevice");
    return fetch(b);
}

int mesh_batch_outputs(mesh_batch *b, void **verts, int64_t **faces, int64_t **offsets) {
    if (!b || !verts || !faces || !offsets) return MESH_EINVAL;
    if (!b->counted) return fail(b->ctx, MESH_ESTATE, "mesh_batch_outputs without mesh_batch_count");
    *verts = b->weld ? b->wv.ptr : b->out_v.ptr;
    *faces = (int64_t *)b->out_f.ptr;
    *offsets = (int64_t *)(b->weld ? b->woffs.ptr : b->offs.ptr);
    return MESH_OK;
}

int mesh_batch_set_graph(mesh_batch *b, int enable) {
    if (!b) return MESH_EINVAL;
    b->use_graph = enable ? 1 : 0;
    if (!enable) drop_graph(b);
    return MESH_OK;
}

int mesh_batch_set_knobs(mesh_batch *b, const int *knobs) {
    if (!b || !knobs) return MESH_EINVAL;
    if (knobs[0] < 0 || knobs[1] < 0 || knobs[2] < 0 || knobs[3] < 96 || knobs[3] > 1024 || knobs[3] % 32)
        return fail(b->ctx, MESH_EINVAL, "knobs out of range");
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return fail(b->ctx, MESH_ECUDA, "cudaSetDevice");
    const int rezone = knobs[0] != b->zs;
    b->zs = knobs[0];
    b->cls_ctas = knobs[1];
    b->cmp_ctas = knobs[2];
    b->scan_threads = knobs[3];
    drop_graph(b);
    if (rezone) return build_plan(b);  // the caller counts again
    return MESH_OK;
}

int mesh_batch_knobs(const mesh_batch *b, int *knobs) {
    if (!b || !knobs) return MESH_EINVAL;
    knobs[0] = b->zs;
    knobs[1] = b->cls_ctas;
    knobs[2] = b->cmp_ctas;
    knobs[3] = b->scan_threads;
    return MESH_OK;
}

int mesh_batch_tune(mesh_batch *b, int reps, char *report, int report_len) {
    if (!b || reps < 1) return MESH_EINVAL;
    mesh_ctx *c = b->ctx;
    c->msg.clear();
    if (cudaSetDevice(c->device) != cudaSuccess) return fail(c, MESH_ECUDA, "cudaSetDevice");
    std::string rep;
    int cur[4] = {b->zs, b->cls_ctas, b->cmp_ctas, b->scan_threads};
    const std::vector<int> cand[4] = {{0, 64, 32, 16}, {0, 2, 1}, {0, 2, 1}, {1024, 512, 256}};
    const char *names[4] = {"zs", "classify_ctas", "compact_ctas", "scan_threads"};
    double best_ms = -1;
    int rc;
    for (int k = 0; k < 4; k++) {
        int best = cur[k];
        for (int val : cand[k]) {
            int kn[4] = {cur[0], cur[1], cur[2], cur[3]};
            kn[k] = val;
            if ((rc = mesh_batch_set_knobs(b, kn)) || (rc = count(b))) return rc;
            double ms = 0;
            if ((rc = time_runs(b, reps, &ms))) return rc;
            char line[128];
            snprintf(line, sizeof(line), "%s=%d %.4f ms\n", names[k], val, ms);
            rep += line;
            if (best_ms < 0 || ms < best_ms) {
                best_ms = ms;
                best = val;
            }
        }
        cur[k] = best;
    }
    if ((rc = mesh_batch_set_knobs(b, cur)) || (rc = count(b))) return rc;
    char line[160];
    snprintf(line, sizeof(line), "best zs=%d classify_ctas=%d compact_ctas=%d scan_threads=%d %.4f ms\n", cur[0],
             cur[1], cur[2], cur[3], best_ms);
    rep += line;
    if (report && report_len > 0) {
        strncpy(report, rep.c_str(), (size_t)report_len - 1);
        report[report_len - 1] = 0;
    }
    return MESH_OK;
}

}  // extern "C"
