#!/usr/bin/env python3
"""Benchmark of the isosurface hot path.

Workload (one step): plain MarchingCubes(iso=0f0) on a 1024^3 Float32 volume
f = sum_{k=1..16} a_k sin(2pi w_k.p + phi_k) over [0,1]^3 (X = Y = Z = 0:1,
seeded a_k ~ N(0,1), |w_k| ~ U[1,8] with a random direction, phi_k ~ U[0,2pi)).
The volume is 4 GiB, larger than L2, so no flush is needed between steps.

Metric: Gvoxels/s counting input samples nx*ny*nz.
  value  -- device-resident: mesh_extract_device (classify -> scan ->
            compaction of the active cells -> expansion into vertices and
            faces) with the volume and preallocated outputs in HBM;
  e2e    -- the two-phase drop-in call (mesh_count + mesh_fill) with pinned
            host buffers: upload, extraction and download of the mesh.
The roofline object reports the dominant kernel's algorithmic bytes over its
CUDA-event time; `pipeline` reports in+out bytes over the whole step.

On one GPU the same JSON line also carries the suite's other workloads, each
with its own clock record (`--no-extras` leaves them out; `--workload X` runs
one of them alone):
  batched -- 4096 uneven Float32 volumes in one tuned, graph-replayed batch,
             against a loop of per-volume calls;
  serving -- Poisson arrivals of mixed requests (32^3..512^3, Float32/Float64,
             60/30/10 MC/MT/NSN) under a 120 GB budget on 6 slots, the offered rate
             doubled until the loop saturates; 128^3 MC requests against a
             batch of the same 256 distinct volumes;
  gyroid  -- MC, MT and NSN on the Float32 256^3 gyroid;
  ct      -- MC on the UInt16 512^3 CT-like volume.

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement of Meshing.jl's MarchingCubes (single-threaded, as the
reference is) on a z slab from the middle of the same field; the in-line
cpu_baseline times the same slab.
Multi-GPU (torchrun): independent replicas, weak scaling.
"""
import argparse
import ctypes
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 1024
SEED = 0
WORKLOAD = ('MarchingCubes(iso=0f0) on a %d^3 Float32 16-term random-sines field over [0,1]^3 '
            '(X=Y=Z=0:1), Julia column-major layout')


def sines_host(n, z0, nz, seed=SEED):
    """numpy version of meshing_gb300.fields.sines for a z slab: C-ordered (nz, n, n) float32."""
    import meshing_gb300.fields as fields  # noqa: F401  (parameters only)
    g = np.linspace(0.0, 1.0, n)
    out = np.zeros((nz, n, n), np.float32)
    for a, w, ph in fields.sines_params(seed):
        ex = np.exp(1j * (2 * np.pi * w[0]) * g).astype(np.complex64)
        ey = np.exp(1j * (2 * np.pi * w[1]) * g).astype(np.complex64)
        ez = np.exp(1j * ((2 * np.pi * w[2]) * g[z0:z0 + nz] + ph)).astype(np.complex64)
        exy = ey[:, None] * ex[None, :]
        for k in range(nz):
            out[k] += np.float32(a) * (ez[k] * exy).imag
    return out


def sines_device(n, seed=SEED, device='cuda'):
    """The benchmark field on the device, Julia layout (x fastest), float32."""
    import torch
    import meshing_gb300.fields as fields
    g = torch.linspace(0.0, 1.0, n, dtype=torch.float64, device=device)
    out = torch.zeros((n, n, n), dtype=torch.float32, device=device)
    zc = 64
    for a, w, ph in fields.sines_params(seed):
        ax = ((2 * math.pi * w[0]) * g).float()
        ay = ((2 * math.pi * w[1]) * g).float()
        az = ((2 * math.pi * w[2]) * g + ph).float()
        for z0 in range(0, n, zc):
            arg = az[z0:z0 + zc, None, None] + ay[None, :, None] + ax[None, None, :]
            out[z0:z0 + zc].add_(torch.sin(arg), alpha=float(a))
    return out.permute(2, 1, 0)


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile('w+', suffix='.csv', delete=False)
        try:
            self.p = subprocess.Popen(['nvidia-smi', '-i', str(index), '--query-gpu=' + self.Q, '--format=csv,noheader',
                                       '-lms', '50'], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        # start timing only once sampling runs
        t0 = time.time()
        while self.p is not None and time.time() - t0 < 5 and os.path.getsize(self.f.name) == 0:
            time.sleep(0.01)

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(',') for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            try:
                sm.append(float(r[1].split()[0]))
                mx = float(r[2].split()[0])
                for nm, v in zip(names, r[5:9]):
                    if 'Active' in v and 'Not' not in v:
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': mx, 'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peak():
    try:
        j = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
        return float(j['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def pieces(nx, ny, nz, sms):
    """Pieces (one z segment of one cell column) of a volume: the engine's tiling rule
    (mesh_api.cu, prepare): 31 x 4-cell warp tiles, z segments of whole 8-cell chunks,
    about 64 warp tiles per SM in all."""
    cx, cy, cz = nx - 1, ny - 1, nz - 1
    per_seg = ((cx + 30) // 31) * ((cy + 3) // 4)
    nseg = min((cz + 7) // 8, max(1, (sms * 64 + per_seg - 1) // per_seg))
    zs = (cz + nseg - 1) // nseg
    zs = (zs + 7) // 8 * 8
    return ((cz + zs - 1) // zs) * cy * cx


def max_over_ranks(dist, values, device='cpu'):
    """Each value's maximum over the ranks: the slowest replica sets the job's time
    (identity without a process group)."""
    if not dist:
        return list(values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(units_per_rank, world, ms):
    """Units per second of the whole job: every replica processes units_per_rank in
    the slowest replica's ms."""
    return units_per_rank * world / (ms * 1e-3)


def _spread(xs):
    """min / median / p90 / max / mean of a list of step times (ms)."""
    if not xs:
        return None
    ys = sorted(xs)
    q = lambda f: ys[min(len(ys) - 1, int(f * len(ys)))]
    return {'min': ys[0], 'median': q(0.5), 'p90': q(0.9), 'max': ys[-1], 'mean': sum(ys) / len(ys)}


def host_link(hvol, hv, hf, dev):
    """Copy-engine throughput (GB/s) of the end-to-end run's own pinned buffers: the
    volume up, the mesh down; best of 3, CUDA events."""
    import torch
    dvol = torch.empty(hvol.shape, dtype=hvol.dtype, device=dev)
    dv = torch.empty(hv.shape, dtype=hv.dtype, device=dev)
    df = torch.empty(hf.shape, dtype=hf.dtype, device=dev)
    out = {}
    for key, pairs in (('h2d_gbs', ((dvol, hvol),)), ('d2h_gbs', ((hv, dv), (hf, df)))):
        nbytes = sum(src.numel() * src.element_size() for _, src in pairs)
        best = None
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for dst, src in pairs:
                dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[key] = nbytes / (best * 1e-3) / 1e9
    del dvol, dv, df
    return out


def host_cpu():
    """CPU model and core count of this host, and whether Julia (Meshing.jl's
    language) is installed."""
    model = None
    try:
        out = subprocess.run(['lscpu'], capture_output=True, text=True, timeout=10).stdout
        fields = dict((a.strip(), b.strip()) for a, b in (ln.split(':', 1) for ln in out.splitlines() if ':' in ln))
        model = fields.get('Model name') or fields.get('Vendor ID')
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open('/proc/cpuinfo'):
                if line.lower().startswith('model name'):
                    model = line.split(':', 1)[1].strip()
                    break
        except OSError:
            pass
    julia = shutil.which('julia')
    return {'cpu_model': model or 'unknown', 'host_cores': os.cpu_count(),
            'meshing_jl': ('julia found at %s (not used: the restatement is timed)' % julia) if julia else
            'Meshing.jl: unavailable on this box (no Julia)'}


# The CPU sample: CPU_PLANES z cell planes from the middle of the benchmark
# volume, the same slab for the reference arm and the in-line cpu_baseline.
CPU_PLANES = 96


def cpu_slab(n, planes):
    """Fortran view (n, n, planes + 1) of z planes from the middle of the field."""
    z0 = max(0, (n - (planes + 1)) // 2)
    slab = sines_host(n, z0, planes + 1)         # C-ordered (nz, n, n) == Julia layout (n, n, nz)
    return slab.transpose(2, 1, 0), z0


def cpu_baseline(n, planes, steps=1, warmup=0, threads=1):
    """Oracle (CPU restatement of MarchingCubes) on a z slab of the field: Gvoxels/s.
    threads > 1 splits the slab into x windows meshed on that many threads."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle
    A, z0 = cpu_slab(n, planes)
    # the slab's z coordinates are its own LinRange nodes, which changes vertex
    # positions only, not the work done
    rng = ((0, 1), (0, 1), (0, 1))
    if threads > 1:
        A = np.asfortranarray(A)
        run = lambda: oracle.mc_xwindows(A, np.float32(0), rng, windows=4 * threads, threads=threads)
    else:
        run = lambda: oracle.isosurface(A, 'mc', np.float32(0), 1e-3, rng)
    for _ in range(warmup):
        run()
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        run()
        times.append(time.perf_counter() - t0)
    dt = sum(times) / len(times)
    vox = float(n) * n * (planes + 1)
    return vox / dt / 1e9, dt, vox, z0


def cpu_sample_text(n, planes, z0, dt, threads):
    return ('z slab %dx%dx%d (planes %d..%d, %.0f M samples) of the benchmark field, CPU restatement of '
            'MarchingCubes (oracle/oracle.c; %s), %.2f s per pass' % (
                n, n, planes + 1, z0, z0 + planes, n * n * (planes + 1) / 1e6,
                'single-threaded like Meshing.jl' if threads == 1 else
                'x windows on %d threads' % threads, dt))


def run_reference(args, rank, world):
    if rank != 0:
        return
    planes = args.cpu_planes or CPU_PLANES
    val, dt, vox, z0 = cpu_baseline(args.n, planes, steps=args.steps, warmup=args.warmup)
    info = host_cpu()
    line = {'impl': 'reference', 'metric': 'Gvoxels/s (input samples per second), plain MarchingCubes',
            'value': val, 'unit': 'Gvoxels/s', 'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': dt * 1e3, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
            'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': WORKLOAD % args.n, 'sample_planes': planes + 1, 'sample_z0': z0},
            'cpu_baseline': {'value': val, 'unit': 'Gvoxels/s', 'cores': 1, 'kind': 'port',
                             'sample': cpu_sample_text(args.n, planes, z0, dt, 1), **info},
            'e2e': {'value': val, 'unit': 'Gvoxels/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    lib = pkg.load_library()
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    n = args.n
    vol = sines_device(n, device=dev)
    torch.cuda.synchronize()
    m = pkg.MarchingCubes(iso=np.float32(0))
    X = Y = Z = (0, 1)
    ctx = pkg.Context(local)
    stream = torch.cuda.current_stream(dev)
    ctx.follow_torch(dev)  # the timing events are recorded on this stream
    p = pkg.make_params(m, X, Y, Z)
    nv, nf = ctypes.c_int64(), ctypes.c_int64()
    pkg._lib.check(lib.mesh_count(ctx.handle, ctypes.c_void_p(vol.data_ptr()), 2, n, n, n, 1, ctypes.byref(p),
                                  ctypes.byref(nv), ctypes.byref(nf)), ctx.handle)
    nv, nf = nv.value, nf.value
    verts = torch.empty((nv, 3), dtype=torch.float32, device=dev)
    faces = torch.empty((nf, 3), dtype=torch.int64, device=dev)
    counts = torch.zeros(2, dtype=torch.int64, device=dev)

    def step():
        pkg._lib.check(lib.mesh_extract_device(ctx.handle, ctypes.c_void_p(vol.data_ptr()), 2, n, n, n,
                                               ctypes.byref(p), ctypes.c_void_p(verts.data_ptr()), nv,
                                               ctypes.c_void_p(faces.data_ptr()), nf,
                                               ctypes.c_void_p(counts.data_ptr())), ctx.handle)

    for _ in range(args.warmup):
        step()
    ctx.sync()
    ctx.stage_times()  # reset
    ctx.enable_timing(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local) if rank == 0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop() if clocks else None
    ctx.sync()
    ms = e0.elapsed_time(e1) / args.steps
    st = ctx.stage_times()
    ctx.enable_timing(False)
    assert counts.tolist() == [nv, nf]

    # end to end through the drop-in C ABI with pinned host buffers
    hvol = torch.empty((n, n, n), dtype=torch.float32, pin_memory=True)
    hvol.copy_(vol.permute(2, 1, 0))
    hv = torch.empty((nv, 3), dtype=torch.float32, pin_memory=True)
    hf = torch.empty((nf, 3), dtype=torch.int64, pin_memory=True)
    ctx.set_stream(None)

    split = []  # per step: (mesh_count ms, mesh_fill ms), host clock

    def e2e_step():
        a, b = ctypes.c_int64(), ctypes.c_int64()
        t0 = time.perf_counter()
        pkg._lib.check(lib.mesh_count(ctx.handle, ctypes.c_void_p(hvol.data_ptr()), 2, n, n, n, 0, ctypes.byref(p),
                                      ctypes.byref(a), ctypes.byref(b)), ctx.handle)
        t1 = time.perf_counter()
        pkg._lib.check(lib.mesh_fill(ctx.handle, ctypes.c_void_p(hv.data_ptr()), ctypes.c_void_p(hf.data_ptr()), 0),
                       ctx.handle)
        split.append(((t1 - t0) * 1e3, (time.perf_counter() - t1) * 1e3))

    for _ in range(max(1, args.warmup)):
        e2e_step()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    split.clear()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    ok = torch.equal(hv.to(dev), verts) and torch.equal(hf.to(dev), faces)
    link = host_link(hvol, hv, hf, dev)  # overwrites hv / hf: after the check

    ms, e2e_ms = max_over_ranks(dist, [ms, e2e_ms], dev)
    # the other workloads of the benchmark suite, each with its own clock record
    # (one GPU only: replicas of a scaling run time the headline alone)
    extras = {}
    if world == 1 and not args.no_extras:
        ctx.close()
        del hvol, hv, hf, vol, verts, faces, counts
        torch.cuda.empty_cache()
        for key, fn in (('batched', measure_batched), ('serving', measure_serving), ('gyroid', measure_gyroid),
                        ('ct', measure_ct)):
            t0 = time.time()
            try:
                extras[key] = fn(args, rank, world, dev)
            except Exception as e:  # a failed side workload is reported, the headline stands
                extras[key] = {'error': '%s: %s' % (type(e).__name__, e)}
            print('bench: %s took %.1f s' % (key, time.time() - t0), file=sys.stderr, flush=True)
    if rank != 0:
        return
    vox = float(n) ** 3
    peak, peak_kind = measured_peak()
    in_b = vox * 4
    out_b = nv * 12 + nf * 24
    stage = {k: v[0] / args.steps for k, v in st.items()}  # each timed step runs every stage once
    # algorithmic bytes per launch (input 4 B per sample, mesh 12 B per vertex and
    # 24 B per face): classify reads every sample (k_classify_tma_mc, staged by
    # TMA, for volumes with 16-byte aligned rows; the load walk k_classify with
    # MESHING_GB300_TMA=0); the scan reads 3
    # u32 counts and writes 3 int64 bases per piece; the direct emission
    # (k_direct_mc) writes the mesh (its second read of the samples of active
    # cells is not algorithmic and is not counted).  In the list form
    # (MESHING_GB300_LIST_EMIT=1) the compaction (k_compact_mc) reads the
    # samples of the active chunks and writes the list of active cells, and the
    # expansion (k_expand_mc) writes the mesh: only the expansion gets bytes.
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    kern = {
        'classify': {'ms': stage['classify'], 'bytes': in_b,
                     'kernel': 'k_classify' if os.environ.get('MESHING_GB300_TMA') == '0' else 'k_classify_tma_mc'},
        'scan': {'ms': stage['scan'], 'bytes': float(pieces(n, n, n, sms) * 3 * (4 + 8)), 'kernel': 'k_scan'},
    }
    if stage.get('expand'):
        kern['compact'] = {'ms': stage['emit'], 'bytes': None, 'kernel': 'k_compact_mc',
                           'note': 'reads the samples of active chunks, writes the active-cell list'}
        kern['expand'] = {'ms': stage['expand'], 'bytes': float(out_b), 'kernel': 'k_expand_mc'}
    else:
        kern['emit'] = {'ms': stage['emit'], 'bytes': float(out_b), 'kernel': 'k_direct_mc',
                        'note': 'writes the mesh; its read of the samples of active cells is not counted'}
    for k in kern.values():
        k['gbs'] = k['bytes'] / (k['ms'] * 1e-3) / 1e9 if k['ms'] and k['bytes'] else None
        k['frac'] = k['gbs'] / peak if k['gbs'] else None
    # the dominant kernel: the longest launch of the step (that has algorithmic bytes)
    dom = max((k for k in kern if kern[k]['bytes']), key=lambda k: kern[k]['ms'])
    achieved = kern[dom]['gbs']
    traffic = None
    tpath = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get('%s_%d' % (dom, n))
        except ValueError:
            traffic = None
    pipe_gbs = (in_b + out_b) / (ms * 1e-3) / 1e9
    cpu = None
    if world == 1 and not args.no_cpu:
        # the reference arm's slab, passes repeated to about 10-30 s of CPU work
        planes = args.cpu_planes or CPU_PLANES
        cval, cdt, _, z0 = cpu_baseline(n, planes, steps=args.cpu_passes)
        cpu = {'value': cval, 'unit': 'Gvoxels/s', 'cores': 1, 'kind': 'port',
               'sample': cpu_sample_text(n, planes, z0, cdt, 1) + ', mean of %d passes' % args.cpu_passes,
               **host_cpu()}
        threads = os.cpu_count() or 1
        if threads > 1:
            pval, pdt, _, _ = cpu_baseline(n, planes, steps=2, threads=threads)
            cpu['all_cores'] = {'value': pval, 'unit': 'Gvoxels/s', 'cores': threads,
                                'sample': cpu_sample_text(n, planes, z0, pdt, threads),
                                'note': 'Meshing.jl itself is single-threaded; this is the restatement split '
                                        'into x windows, for scale'}
    line = {
        'metric': 'Gvoxels/s (input samples per second), plain MarchingCubes',
        'value': whole_job_rate(vox, world, ms) / 1e9,
        'unit': 'Gvoxels/s', 'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': WORKLOAD % n, 'nx': n, 'ny': n, 'nz': n, 'cells': (n - 1) ** 3, 'nverts': nv,
                   'nfaces': nf, 'output': 'Float32 vertices, Int64 1-based faces', 'l2': 'inputs larger than L2',
                   'parallelism': 'replicas' if world > 1 else 'single GPU',
                   'stage_ms': stage, 'e2e_matches_device': bool(ok)},
        'roofline': {'bound': 'hbm', 'kernel': dom, 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': traffic, 'peak_source': peak_kind,
                     'algorithmic_bytes': kern[dom]['bytes']},
        'kernels': kern,
        'pipeline': {'bytes': in_b + out_b, 'achieved': pipe_gbs, 'frac': pipe_gbs / peak, 'unit': 'GB/s'},
        'e2e': {'value': whole_job_rate(vox, world, e2e_ms) / 1e9, 'unit': 'Gvoxels/s', 'ms_per_step': e2e_ms,
                'h2d_bytes_per_step': int(in_b), 'd2h_bytes_per_step': int(out_b),
                'count_ms': _spread([c for c, _ in split]), 'fill_ms': _spread([f for _, f in split]),
                'step_ms': _spread([c + f for c, f in split]),
                'link': link, 'link_bound_ms': (in_b / link['h2d_gbs'] + out_b / link['d2h_gbs']) / 1e6},
        'gpu_launches': int(sum(v[1] for v in st.values())),
        'cpu_baseline': cpu,
        'clocks': ck,
    }
    e = line['e2e']
    e['median_over_link_bound'] = e['step_ms']['median'] / e['link_bound_ms']
    line.update(extras)
    print(json.dumps(line), flush=True)


def measure_batched(args, rank, world, dev):
    """The batched workload: MarchingCubes(iso=0f0) on `--volumes` Float32
    volumes, each axis 16..128, min-union SDFs of 1-8 seeded spheres / boxes on
    [-1,1]^3.  value: one batch (tuned knobs, replayed from a CUDA graph); the
    loop line: the same volumes through one mesh_extract_device call each."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import meshing_gb300.fields as fields
    lib = pkg.load_library()
    local = dev.index or 0
    vols = fields.batch_volumes(args.volumes, seed=SEED + rank, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    nv, nf = b.count()
    report = b.tune(reps=3)
    b.set_graph(True)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        b.run()
    b.sync()
    clocks = Clocks(local) if rank == 0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.run()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop() if clocks else None
    b.sync()
    ms = e0.elapsed_time(e1) / args.steps
    verts, faces, offs = b.outputs()
    o = offs.cpu().numpy()
    # a loop of plain per-volume launches into the same layout
    ctx = b.ctx
    p = pkg.make_params(m, (-1, 1), (-1, 1), (-1, 1))
    lv, lf = torch.empty_like(verts), torch.empty_like(faces)
    cnt = torch.zeros((len(vols), 2), dtype=torch.int64, device=dev)
    jl = [pkg.api._torch_julia_layout(v) for v in vols]

    def loop():
        for i, t in enumerate(jl):
            pkg._lib.check(lib.mesh_extract_device(
                ctx.handle, ctypes.c_void_p(t.data_ptr()), 2, t.shape[0], t.shape[1], t.shape[2], ctypes.byref(p),
                ctypes.c_void_p(lv.data_ptr() + 12 * int(o[i, 0])), int(o[i + 1, 0] - o[i, 0]),
                ctypes.c_void_p(lf.data_ptr() + 24 * int(o[i, 1])), int(o[i + 1, 1] - o[i, 1]),
                ctypes.c_void_p(cnt[i].data_ptr())), ctx.handle)

    loop()
    torch.cuda.synchronize()
    lsteps = max(1, min(args.steps, 3))
    e0.record(stream)
    for _ in range(lsteps):
        loop()
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1) / lsteps
    same = torch.equal(lv, verts) and torch.equal(lf, faces)
    vox = float(sum(v.numel() for v in vols))
    in_b, out_b = vox * 4, nv * 12 + nf * 24
    peak, peak_kind = measured_peak()
    gbs = (in_b + out_b) / (ms * 1e-3) / 1e9
    knobs = b.knobs
    del jl, lv, lf, verts, faces, offs
    b.close()
    del vols
    torch.cuda.empty_cache()
    return {
        'metric': 'Gvoxels/s (input samples per second), batched MarchingCubes', 'workload': 'batched',
        'value': vox * world / (ms * 1e-3) / 1e9, 'unit': 'Gvoxels/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic',
        'config': {'workload': '%d Float32 volumes, each axis uniform in 16..128, min-union SDF of 1-8 seeded spheres '
                               '/ boxes on [-1,1]^3, MarchingCubes(iso=0f0)' % args.volumes,
                   'volumes': args.volumes, 'samples': int(vox), 'nverts': nv, 'nfaces': nf, 'knobs': knobs,
                   'graph': True, 'l2': 'inputs larger than L2'},
        'loop': {'value': vox / (loop_ms * 1e-3) / 1e9, 'ms_per_step': loop_ms, 'steps': lsteps,
                 'what': 'one mesh_extract_device call per volume, same stream, same outputs',
                 'identical_outputs': bool(same)},
        'speedup_vs_loop': loop_ms / ms,
        'pipeline': {'bytes': in_b + out_b, 'achieved': gbs, 'peak': peak, 'frac': gbs / peak, 'unit': 'GB/s',
                     'peak_source': peak_kind},
        'tuner': report.strip().splitlines()[-1],
        'clocks': ck,
    }


def run_batched(args, rank, world):
    import torch
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    line = measure_batched(args, rank, world, torch.device('cuda', local))
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_serving(args, rank, world, dev):
    """The serving workload: Poisson arrivals of requests whose cubic size is
    log-uniform in 32..512, 50/50 Float32 / Float64, fields of the plain
    (random sines on [0,1]^3) and batched (primitive SDFs on [-1,1]^3)
    generators, 60/30/10 MarchingCubes / MarchingTetrahedra / NaiveSurfaceNets,
    answered by the serving loop under a device-memory budget and a bounded
    queue.  The offered rate doubles from --rate0 until the loop saturates
    (served below 90% of offered, or requests rejected) and one rate past that.
    Then 128^3 MarchingCubes requests over 256 distinct volumes of the batched
    generator, against one graph-replayed batch of the same 256 volumes."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import meshing_gb300.fields as fields
    local = dev.index or 0
    rng = np.random.default_rng(SEED + rank)
    pool = []
    for k in range(args.pool):
        n = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
        dt = torch.float32 if k % 2 == 0 else torch.float64
        if rng.random() < 0.5:
            pool.append((fields.sines(n, seed=k, dtype=dt, device=dev), ((0, 1),) * 3))
        else:
            pool.append((fields.primitives_sdf((n, n, n), fields.primitives_params(rng), dtype=dt, device=dev),
                         ((-1, 1),) * 3))
    torch.cuda.synchronize()

    def method(a, dt):
        iso = np.float32(0) if dt == torch.float32 else 0.0
        return [pkg.MarchingCubes, pkg.MarchingTetrahedra, pkg.NaiveSurfaceNets][a](iso=iso)

    srv = pkg.Server(budget_bytes=int(args.budget_gb * 1e9), slots=args.slots, max_wave=256, max_queue=args.max_queue,
                     device=local)
    # warm-up (pinned staging, context scratch, kernel caches), not measured
    warm = [(A, method(a, A.dtype), r) for A, r in pool for a in range(3)]
    srv.replay(warm, np.zeros(len(warm)))
    clocks = Clocks(local) if rank == 0 else None
    sweep = []
    rate, past = args.rate0, 0
    while len(sweep) < args.max_rates and past < 2:
        nreq = int(min(args.requests, max(200, rate * 3)))
        reqs = []
        for _ in range(nreq):
            A, r = pool[int(rng.integers(len(pool)))]
            reqs.append((A, method(int(rng.choice(3, p=[0.6, 0.3, 0.1])), A.dtype), r))
        arr = np.cumsum(rng.exponential(1.0 / rate, nreq))
        srv.reset_stats()
        t0 = time.time()
        srv.replay(reqs, arr)
        st = srv.stats()
        print('serving mixed %.0f/s: %d requests in %.1f s, %.1f per wave' % (
            rate, nreq, time.time() - t0, st['requests_per_wave']), file=sys.stderr, flush=True)
        thr = st['completed'] / st['wall_s'] if st['wall_s'] else 0
        sweep.append({'offered_per_s': rate, 'requests': nreq, 'completed': int(st['completed']),
                      'rejected': int(st['rejected']), 'failed': int(st['failed']),
                      'rejection_rate': st['rejected'] / nreq,
                      'throughput_per_s': thr,
                      'gvox_per_s': st['samples'] / st['wall_s'] / 1e9 if st['wall_s'] else 0,
                      'p50_ms': st['p50_ms'], 'p99_ms': st['p99_ms'], 'mean_ms': st['mean_ms'],
                      'peak_reserved_gb': st['peak_reserved_bytes'] / 1e9,
                      'requests_per_wave': st['requests_per_wave']})
        if past or st['rejected'] > 0 or thr < 0.9 * rate:
            past += 1
        rate *= 2
    del pool, warm, reqs
    ck_mixed = clocks.stop() if clocks else None
    torch.cuda.empty_cache()

    # 128^3 Marching Cubes requests: the serving loop against one batch of the same volumes
    nvol = 256
    vols = [fields.primitives_sdf((128, 128, 128), fields.primitives_params(rng), dtype=torch.float32, device=dev)
            for _ in range(nvol)]
    m = pkg.MarchingCubes(iso=np.float32(0))
    b = pkg.Batch(vols, m)
    b.count()
    b.set_graph(True)
    for _ in range(3):
        b.run()
    b.sync()
    clocks = Clocks(local) if rank == 0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(10):
        b.run()
    e1.record()
    torch.cuda.synchronize()
    batched = nvol * 128 ** 3 / (e0.elapsed_time(e1) / 10 * 1e-3) / 1e9
    b.close()
    uniform = []
    srv.replay([(v, m, ((-1, 1),) * 3) for v in vols], np.zeros(nvol))  # warm-up, not measured
    for rate in [float(x) for x in args.rates128.split(',')]:
        nreq = int(min(args.requests128, max(200, rate * 2)))
        reqs = [(vols[int(rng.integers(nvol))], m, ((-1, 1),) * 3) for _ in range(nreq)]
        arr = np.cumsum(rng.exponential(1.0 / rate, nreq))
        srv.reset_stats()
        t0 = time.time()
        srv.replay(reqs, arr)
        st = srv.stats()
        print('serving 128^3 %.0f/s: %d requests in %.1f s, %.1f per wave' % (
            rate, nreq, time.time() - t0, st['requests_per_wave']), file=sys.stderr, flush=True)
        g = st['samples'] / st['wall_s'] / 1e9 if st['wall_s'] else 0
        uniform.append({'offered_per_s': rate, 'requests': nreq, 'completed': int(st['completed']),
                        'rejected': int(st['rejected']), 'rejection_rate': st['rejected'] / nreq,
                        'throughput_per_s': st['completed'] / st['wall_s'] if st['wall_s'] else 0,
                        'gvox_per_s': g, 'fraction_of_batched': g / batched, 'p50_ms': st['p50_ms'],
                        'p99_ms': st['p99_ms'], 'requests_per_wave': st['requests_per_wave']})
    ck_128 = clocks.stop() if clocks else None
    srv.close()
    del vols, reqs
    torch.cuda.empty_cache()
    best = max(sweep, key=lambda x: x['gvox_per_s'])
    ok128 = [u for u in uniform if u['p99_ms'] < 10.0 and u['rejected'] == 0]
    return {
        'metric': 'Gvoxels/s (input samples per second), serving loop', 'workload': 'serving',
        'value': best['gvox_per_s'], 'unit': 'Gvoxels/s', 'n_gpus': world, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32/f64', 'data': 'synthetic',
        'config': {'workload': 'Poisson arrivals; cubic sizes log-uniform 32..512; 50/50 Float32 / Float64; random '
                               'sines on [0,1]^3 or primitive SDFs on [-1,1]^3; 60/30/10 MC / MT / NSN; iso 0',
                   'budget_gb': args.budget_gb, 'slots': args.slots, 'max_wave': 256, 'max_queue': args.max_queue,
                   'volume_pool': args.pool},
        'sweep': sweep,
        'saturation_per_s': max(x['throughput_per_s'] for x in sweep),
        'clocks': ck_mixed,
        'uniform_128_mc': {'batched_gvox_per_s': batched,
                           'batched_what': '%d distinct 128^3 Float32 volumes of the batched generator (min-union '
                                           'SDFs of 1-8 spheres / boxes), one graph-replayed batch' % nvol,
                           'requests_over': 'the same %d volumes, drawn uniformly' % nvol,
                           'points': uniform,
                           'best_fraction_with_p99_under_10ms': max((u['fraction_of_batched'] for u in ok128),
                                                                    default=None),
                           'clocks': ck_128},
    }


def run_serving(args, rank, world):
    import torch
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    line = measure_serving(args, rank, world, torch.device('cuda', local))
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_ct(args, rank, world, dev):
    """MarchingCubes(iso=500) on the UInt16 512^3 CT-like volume: background
    N(100, 20) clamped to >= 0 plus 3 seeded ellipsoidal shells N(1000, 50), 4
    voxels thick (X = Y = Z = -1:1; UInt16 differences wrap).  Device time per
    call through mesh_extract_device, per stage, and the roofline of each kernel."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import meshing_gb300.fields as fields
    n = args.n if args.n != N_DEFAULT else 512
    t = fields.ct_like_u16(n, seed=SEED, device=dev)
    torch.cuda.synchronize()
    m = pkg.MarchingCubes(iso=500)
    ctx = pkg.Context(dev.index or 0)
    v, f = pkg.isosurface(t, m, ctx=ctx)
    verts, faces = torch.empty_like(v), torch.empty_like(f)
    for _ in range(args.warmup):
        pkg.isosurface_device(t, m, verts=verts, faces=faces, ctx=ctx)
    ctx.sync()
    ctx.stage_times()
    ctx.enable_timing(True)
    stream = torch.cuda.current_stream()
    clocks = Clocks(dev.index or 0) if rank == 0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        pkg.isosurface_device(t, m, verts=verts, faces=faces, ctx=ctx)
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop() if clocks else None
    ctx.sync()
    ms = e0.elapsed_time(e1) / args.steps
    st = {k: v_[0] / args.steps for k, v_ in ctx.stage_times().items() if v_[1]}
    ok = torch.equal(verts, v) and torch.equal(faces, f)
    ctx.close()
    peak, peak_kind = measured_peak()
    in_b = float(n) ** 3 * 2
    out_b = v.shape[0] * 24 + f.shape[0] * 24  # Float64 vertices (Int ranges, Int iso)
    kern = {'classify': (st.get('classify', 0), in_b)}
    if st.get('expand'):  # list form: compaction, then expansion (writes the mesh)
        kern['expand'] = (st['expand'], out_b)
    else:  # direct emission (writes the mesh)
        kern['emit'] = (st.get('emit', 0), out_b)
    roof = {k: {'ms': t_, 'gbs': b / (t_ * 1e-3) / 1e9 if t_ else None,
                'frac': b / (t_ * 1e-3) / 1e9 / peak if t_ else None} for k, (t_, b) in kern.items()}
    nv, nf = v.shape[0], f.shape[0]
    del t, v, f, verts, faces
    torch.cuda.empty_cache()
    return {'metric': 'Gvoxels/s (input samples per second), plain MarchingCubes', 'workload': 'ct',
            'value': n ** 3 / (ms * 1e-3) / 1e9, 'unit': 'Gvoxels/s', 'ms_per_step': ms, 'steps': args.steps,
            'dtype': 'u16', 'data': 'synthetic',
            'config': {'workload': 'UInt16 %d^3 CT-like volume (N(100,20) background, 3 seeded '
                                   'ellipsoidal shells N(1000,50)), MarchingCubes(iso=500)' % n,
                       'nverts': nv, 'nfaces': nf, 'output': 'Float64 vertices',
                       'stage_ms': st, 'repeatable': bool(ok), 'l2': 'inputs larger than L2'},
            'kernels': roof, 'peak': peak, 'peak_source': peak_kind,
            'pipeline': {'bytes': in_b + out_b, 'frac': (in_b + out_b) / (ms * 1e-3) / 1e9 / peak},
            'clocks': ck}


def run_ct(args, rank, world):
    import torch
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    line = measure_ct(args, rank, world, torch.device('cuda', local))
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_gyroid(args, rank, world, dev):
    """MarchingCubes, MarchingTetrahedra and NaiveSurfaceNets, iso 0, on the
    Float32 gyroid sin x cos y + sin y cos z + sin z cos x over [-3pi, 3pi]^3
    (`--n` nodes per axis, 256 by default here): device time per call and per
    stage through mesh_extract_device."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    import meshing_gb300.fields as fields
    n = args.n if args.n != N_DEFAULT else 256
    t = fields.gyroid(n, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    r = (-3 * math.pi, 3 * math.pi)
    peak, peak_kind = measured_peak()
    out = {}
    for name, m in (('MarchingCubes', pkg.MarchingCubes(iso=0.0)), ('MarchingTetrahedra', pkg.MarchingTetrahedra(iso=0.0)),
                    ('NaiveSurfaceNets', pkg.NaiveSurfaceNets(iso=0.0))):
        ctx = pkg.Context(dev.index or 0)
        v, f = pkg.isosurface(t, m, r, r, r, ctx=ctx)
        verts, faces = torch.empty_like(v), torch.empty_like(f)
        for _ in range(args.warmup):
            pkg.isosurface_device(t, m, r, r, r, verts=verts, faces=faces, ctx=ctx)
        ctx.sync()
        ctx.stage_times()
        ctx.enable_timing(True)
        # the 64 MiB volume fits in L2: every timed call follows a write of a buffer
        # larger than L2, and only the calls are timed (CUDA events around each)
        flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
        clocks = Clocks(dev.index or 0) if rank == 0 else None
        evs = []
        for _ in range(args.steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            pkg.isosurface_device(t, m, r, r, r, verts=verts, faces=faces, ctx=ctx)
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
        ck = clocks.stop() if clocks else None
        ctx.sync()
        ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
        del flush
        st = {k: v[0] / args.steps for k, v in ctx.stage_times().items() if v[1]}
        ok = torch.equal(verts, v) and torch.equal(faces, f)
        # bytes in (Float32 samples) + bytes out (Float64 vertices: the Float64 iso; Int64 faces)
        io = n ** 3 * 4 + v.shape[0] * 24 + f.shape[0] * 24
        out[name] = {'ms_per_call': ms, 'gvox_per_s': n ** 3 / (ms * 1e-3) / 1e9, 'nverts': v.shape[0],
                     'nfaces': f.shape[0], 'stage_ms': st, 'repeatable': bool(ok),
                     'roofline': {'bytes': io, 'achieved': io / (ms * 1e-3) / 1e9,
                                  'frac': io / (ms * 1e-3) / 1e9 / peak, 'unit': 'GB/s'},
                     'clocks': ck}
        ctx.close()
        del v, f, verts, faces
    del t
    torch.cuda.empty_cache()
    return {'metric': 'Gvoxels/s per algorithm', 'workload': 'gyroid', 'n': n, 'dtype': 'f32', 'steps': args.steps,
            'config': {'workload': 'Float32 %d^3 gyroid over [-3pi,3pi]^3, iso 0.0 (Float64)' % n,
                       'l2': 'L2 flushed before every timed call (a 512 MiB write); calls timed one by one'},
            'peak': peak, 'peak_source': peak_kind, 'algorithms': out}


def run_gyroid(args, rank, world):
    import torch
    local = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(local)
    line = measure_gyroid(args, rank, world, torch.device('cuda', local))
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=100)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--n', type=int, default=N_DEFAULT, help='grid size per axis (default 1024)')
    ap.add_argument('--cpu-planes', type=int, default=None,
                    help='z cell planes of the CPU sample (default %d, about 2-3 s per pass on one core)' % CPU_PLANES)
    ap.add_argument('--cpu-passes', type=int, default=6, help='passes over the CPU sample for cpu_baseline')
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    ap.add_argument('--no-extras', action='store_true',
                    help='plain workload only: skip the batched, serving, gyroid and CT results of the default line')
    ap.add_argument('--workload', default='plain', choices=['plain', 'batched', 'serving', 'gyroid', 'ct'],
                    help='plain: one 1024^3 volume (the headline); batched: many uneven volumes; serving: the '
                         'serving loop under Poisson arrivals')
    ap.add_argument('--volumes', type=int, default=4096, help='volumes of the batched workload')
    ap.add_argument('--pool', type=int, default=40, help='serving: distinct resident request volumes')
    ap.add_argument('--budget-gb', type=float, default=120.0, help='serving: device memory budget')
    ap.add_argument('--slots', type=int, default=6, help='serving: waves in flight at once')
    ap.add_argument('--rate0', type=float, default=400.0,
                    help='serving: first offered rate (requests per second); doubled until the loop saturates')
    ap.add_argument('--max-rates', type=int, default=8, help='serving: at most this many offered rates')
    ap.add_argument('--max-queue', type=int, default=1024, help='serving: waiting requests beyond which the loop '
                                                                'rejects (MESH_EBUSY)')
    ap.add_argument('--requests', type=int, default=1500, help='serving: requests per rate (at most)')
    ap.add_argument('--rates128', default='60000,120000,160000,200000,240000',
                    help='serving 128^3: offered requests per second')
    ap.add_argument('--requests128', type=int, default=60000, help='serving 128^3: requests per rate (at most)')
    args = ap.parse_args()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    import __graft_entry__ as ge
    ge.load_package()
    if args.impl == 'reference':
        run_reference(args, rank, world)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
        tdist.init_process_group('nccl')
        dist = tdist
    try:
        if args.workload == 'batched':
            run_batched(args, rank, world)
        elif args.workload == 'serving':
            run_serving(args, rank, world)
        elif args.workload == 'gyroid':
            run_gyroid(args, rank, world)
        elif args.workload == 'ct':
            run_ct(args, rank, world)
        else:
            run_ours(args, rank, world, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == '__main__':
    main()
