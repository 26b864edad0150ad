"""Benchmark: batched Lenia search rollout on the GB300 engine.

Workload (search batch, drop-in for leniax run_scan_mem_optimized): 1024
worlds of 128x128, C=1 K=1, kernel R=13 one ring exp(4 - 1/(r(1-r))), gaussian
growth m=0.15 s=0.015, dt=0.1, 1024 Euler steps, uniform[0,1) 48x48 central
patches scaled by a per-world factor in [0.5, 1] (PCG64 seed 1), per-step
leniax statistics + mass centroid, leniax stop count N and the box stop set.

One bench "step" = one full rollout of that batch (1024 worlds x 1024 Euler
steps).  Metric: cell-updates/s = worlds * cells * Euler steps / time.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) each rank runs its own 1024-world batch (worlds are
independent: weak scaling, no collective on the data path); rank 0 prints the
JSON line with the max time over ranks.
"""
import argparse
import json
import os
import statistics as pystats
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'cell-updates/s'
WORKLOAD = 'search-1024x128x128-c1k1-1024steps'
N_WORLDS, SIZE, STEPS_EULER, PATCH, R, T_RATE = 1024, 128, 1024, 48, 13, 10.0
KPARAMS = [{
    'k_slug': 'circle_2d', 'k_params': [1.0, [1.0]], 'kf_slug': 'gauss_bump', 'kf_params': [1.0], 'gf_slug': 'gaussian',
    'gf_params': [0.15, 0.015], 'h': 1.0, 'c_in': 0, 'c_out': 0
}]
P_CELLS = SIZE * SIZE


def flops_per_world_step(C, K, P, stats=True):
    """Algorithmic flops of one Euler step of one world with P cells per
    channel: r2c + c2r transforms (C + K) * 2.5 P log2 P, spectrum multiply
    6 K (P/2 + 1), growth 8 K P (exp counted as 1), weighting 2 K P, Euler +
    clip 4 C P, statistics 10 C P."""
    f = (C + K) * 2.5 * P * np.log2(P) + 6 * K * (P // 2 + 1) + (8 + 2) * K * P + 4 * C * P
    return f + (10 * C * P if stats else 0)


def adjoint_flops_per_world_step(P):
    """Algorithmic flops of one reverse step of a C = K = 1 world: transforms
    of dL/du and of the state and the inverse of the correlation 3 * 2.5 P
    log2 P, the conjugate-spectrum product and the kernel-gradient
    accumulation 14 (P/2 + 1), the pointwise adjoint (clip gradient, growth
    derivative, parameter partial sums) 20 P."""
    return 3 * 2.5 * P * np.log2(P) + 14 * (P // 2 + 1) + 20 * P


FLOPS_PER_WORLD_STEP = flops_per_world_step(1, 1, P_CELLS)
CPU_SAMPLE_WORLDS, CPU_SAMPLE_STEPS = 64, 320
PLAIN_SAMPLE_WORLDS, PLAIN_SAMPLE_STEPS = 64, 64


def make_inputs(n_worlds, seed=1):
    rng = np.random.Generator(np.random.PCG64(seed))
    cells = np.zeros((1, n_worlds, 1, SIZE, SIZE), np.float32)
    lo = (SIZE - PATCH) // 2
    noise = rng.random((n_worlds, PATCH, PATCH), dtype=np.float32)
    factor = rng.uniform(0.5, 1.0, size=(n_worlds, 1, 1)).astype(np.float32)
    cells[0, :, 0, lo:lo + PATCH, lo:lo + PATCH] = noise * factor
    return cells


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class _OracleSample:
    """The FP32 numpy/scipy restatement of the path (the oracle) on the host
    cores: ``run(steps)`` advances CPU_SAMPLE_WORLDS worlds of the workload
    ``steps`` Euler steps from their initial states (statistics and both stop
    sets included) and returns the seconds it took."""

    def __init__(self):
        from oracle import lenia_oracle as O
        self.O = O
        self.cores = host_cores()
        self.K, mp = O.get_kernels_and_mapping([dict(p) for p in KPARAMS], [SIZE, SIZE], 1, R, True, np.float32)
        self.mp, self.model = mp, O.Model(mp)
        self.cells = make_inputs(CPU_SAMPLE_WORLDS, seed=1)[0]

    def run(self, steps):
        t0 = time.perf_counter()
        self.O.run_scan(self.cells, self.K, self.mp['gf_params'], self.mp['weights'], T_RATE, steps, R, self.model,
                        keep_intermediary=False, workers=self.cores, with_box=True)
        return time.perf_counter() - t0

    def describe(self, steps, seconds):
        return (f'{CPU_SAMPLE_WORLDS} worlds x {steps} steps of the workload (numpy/scipy.fft FP32 restatement, '
                f'scipy workers={self.cores}), {seconds:.1f} s')


def cpu_baseline():
    """The oracle on the host cores, timed on one bounded sample of the
    workload (CPU_SAMPLE_WORLDS worlds x CPU_SAMPLE_STEPS steps)."""
    smp = _OracleSample()
    smp.run(4)
    dt = smp.run(CPU_SAMPLE_STEPS)
    value = CPU_SAMPLE_WORLDS * P_CELLS * CPU_SAMPLE_STEPS / dt
    return {'value': value, 'unit': METRIC, 'cores': smp.cores, 'kind': 'port',
            'sample': smp.describe(CPU_SAMPLE_STEPS, dt)}


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.Q}',
                                          '--format=csv,noheader,nounits', '-lms', '200'], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == 'active':
                    reasons.add(n)
        return {'sm_mhz': pystats.median(sm) if sm else None, 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except Exception:
        return {}


# DRAM bytes (read + write) of the resident kernel, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) on this workload at 1024
# worlds x 64 and x 128 steps and split into a per-world term (state in and
# out) and a per-world-step term (the raw moment record); the bench scales
# them to its own worlds and steps.
# (90.76 MB at 64 steps, 94.26 MB at 128 steps: reads are the 64 KB input
# state of each world; most of the output state is still in L2 when the
# kernel ends).
RESIDENT_DRAM_BYTES_PER_WORLD = 85226.0
RESIDENT_DRAM_BYTES_PER_WORLD_STEP = 53.3


def run_ours(args, rank, world_size):
    import torch
    from leniax_gb300 import _lib, helpers, kernels, runner, statistics

    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    lib = _lib.load()
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in KPARAMS], [SIZE, SIZE], 1, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    stats_fn = statistics.ComputeStatsFn([SIZE, SIZE], R, T_RATE)
    cells_np = make_inputs(N_WORLDS, seed=1 + rank)
    cells = torch.from_numpy(cells_np).to(dev)
    Kb, gf, w = K[None], mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None]
    Tt = torch.tensor([T_RATE], device=dev)

    # device-resident rollout through the engine (inputs already in HBM)
    m = upd.model
    kh = torch.view_as_real(Kb.reshape(1, 1, 1, SIZE, SIZE)[..., :SIZE // 2 + 1].contiguous())
    gfc, wc = gf.contiguous(), w.contiguous()
    final = torch.empty_like(cells)
    st = torch.empty((1, STEPS_EULER, N_WORLDS, 1 + _lib.NSTAT_SCALAR), device=dev)
    ncont = torch.empty((1, N_WORLDS), device=dev)
    nbox = torch.empty((1, N_WORLDS), device=dev)
    cen = torch.empty((1, STEPS_EULER, N_WORLDS, 2), device=dev)
    eng = _lib.ENGINES['auto']
    ws = torch.empty(lib.lgx_run_workspace_bytes(m.plan.handle, 1, N_WORLDS, STEPS_EULER, eng), dtype=torch.uint8,
                     device=dev)
    stream = torch.cuda.current_stream(dev)
    ev_main = [torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
    for e in ev_main:
        e.record(stream)  # materialise the cudaEvent_t handles
    job = _lib.Rollout()
    job.n_sols, job.n_init, job.steps = 1, N_WORLDS, STEPS_EULER
    job.cells0, job.k_half, job.gf_params, job.weights, job.T = (cells.data_ptr(), kh.data_ptr(), gfc.data_ptr(),
                                                                  wc.data_ptr(), Tt.data_ptr())
    job.stats_R, job.stats_T = R, T_RATE
    job.final_cells, job.stats, job.n_continue, job.n_box = (final.data_ptr(), st.data_ptr(), ncont.data_ptr(),
                                                              nbox.data_ptr())
    job.centroid = cen.data_ptr()
    job.engine = eng
    job.main_events[0] = ev_main[0].cuda_event
    job.main_events[1] = ev_main[1].cuda_event
    engine_used = {1: 'resident', 2: 'streamed'}.get(lib.lgx_select_engine(m.plan.handle, 1, N_WORLDS, eng), '?')
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    def rollout():
        _lib.check(lib.lgx_run(m.plan.handle, job, ws.data_ptr(), ws.numel(), stream.cuda_stream))

    for _ in range(args.warmup):
        rollout()
    torch.cuda.synchronize()
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index)
    sampler.start()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    main_ms = []
    for i in range(args.steps):
        flush.zero_()  # L2 flush between timed iterations (outside the timed events)
        evs[i][0].record(stream)
        rollout()
        evs[i][1].record(stream)
        torch.cuda.synchronize()
        main_ms.append(ev_main[0].elapsed_time(ev_main[1]))
    torch.cuda.synchronize()
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = sampler.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in evs)
    if world_size > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    cell_updates = N_WORLDS * P_CELLS * STEPS_EULER
    value = world_size * cell_updates * args.steps / (total_ms / 1e3)
    n_alive = float(nbox.mean().item())

    # roofline of the dominant kernel (FP32-pipe bound)
    kern_ms = pystats.median(main_ms)
    flops_launch = FLOPS_PER_WORLD_STEP * N_WORLDS * STEPS_EULER
    sink = torch.empty(4096, device=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    pb = sms * 8
    lib.lgx_fp32_probe(sink.data_ptr(), pb, 64, stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iters = 4096
    pf = lib.lgx_fp32_probe(sink.data_ptr(), pb, iters, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    fp32_peak = pf / (e0.elapsed_time(e1) / 1e3) / 1e12
    achieved = flops_launch / (kern_ms / 1e3) / 1e12

    # end to end through the public API: pinned host inputs -> device -> rollout -> host results
    host_cells = torch.from_numpy(cells_np).pin_memory()
    e2e_times = []
    h2d = host_cells.numel() * 4  # the batch of initial states; spectra and parameters stay resident
    d2h = 0
    for i in range(max(2, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c_dev = host_cells.to(dev, non_blocking=True)
        sd, fin = runner.run_scan_mem_optimized(None, c_dev, Kb, gf, w, Tt, STEPS_EULER, R, upd, stats_fn,
                                                with_box=True, with_centroid=True)
        outs = [sd['mass'].to('cpu', non_blocking=True), sd['mass_centroid'].to('cpu', non_blocking=True),
                sd['N'].to('cpu', non_blocking=True), sd['N_box'].to('cpu', non_blocking=True),
                fin.to('cpu', non_blocking=True)]
        torch.cuda.synchronize()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
        d2h = sum(o.numel() * 4 for o in outs)
    e2e_value = world_size * cell_updates / pystats.median(e2e_times)

    # plain one-world-per-launch engines on a sample of the same workload: the
    # fused one-kernel step (the resident kernel for one world and one Euler
    # step per launch) and the streamed engine's four-kernel sequence
    sub = cells[:, :PLAIN_SAMPLE_WORLDS].contiguous()
    plain = {}
    for eng in ('plain', 'plain_streamed'):
        runner.run_scan_mem_optimized(None, sub, Kb, gf, w, Tt, 4, R, upd, stats_fn, engine=eng)
        torch.cuda.synchronize()
        ms_plain = _timed(lambda: runner.run_scan_mem_optimized(None, sub, Kb, gf, w, Tt, PLAIN_SAMPLE_STEPS, R, upd,
                                                                stats_fn, engine=eng), stream, flush, 2)
        plain[eng] = PLAIN_SAMPLE_WORLDS * P_CELLS * PLAIN_SAMPLE_STEPS / (ms_plain / 1e3)
    plain_value = plain['plain']

    adjoint = measure_adjoint(dev, fp32_peak=fp32_peak)
    adjoint['variant_3d'] = measure_adjoint_3d(dev)
    multichannel = measure_multichannel(dev, fp32_peak=fp32_peak)
    nd = measure_nd(dev, fp32_peak=fp32_peak)
    uneven = measure_uneven(dev, fp32_peak=fp32_peak)

    gpu_launches = args.steps * 4  # prepare spectrum, resident kernel, stats, heuristics per rollout
    out = {
        'metric': METRIC,
        'value': value,
        'unit': METRIC,
        'n_gpus': world_size,
        'steps': args.steps,
        'warmup': args.warmup,
        'ms_per_step': ms_per_step,
        'higher_is_better': True,
        'scaling': 'weak',
        'vs_baseline': None,
        'dtype': 'f32',
        'data': 'synthetic (PCG64 seeded uniform patches)',
        'config': {
            'workload': WORKLOAD, 'worlds_per_gpu': N_WORLDS, 'world': [SIZE, SIZE], 'channels': 1, 'kernels': 1,
            'euler_steps_per_step': STEPS_EULER, 'engine': engine_used, 'parallelism': f'replicas{world_size}',
            'l2': 'flushed between timed iterations (256 MB write)', 'stats': 'leniax 12 stats + centroid per step',
            'stop_sets': ['leniax check_heuristics', 'box (mass<1e-3, mass>0.9 area, border)'],
            'mean_stop_step_box_set': n_alive
        },
        'e2e': {'value': e2e_value, 'unit': METRIC, 'h2d_bytes_per_step': int(h2d), 'd2h_bytes_per_step': int(d2h)},
        'roofline': {
            'bound': 'fp32', 'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s', 'frac': achieved / fp32_peak,
            'traffic': N_WORLDS * (RESIDENT_DRAM_BYTES_PER_WORLD + RESIDENT_DRAM_BYTES_PER_WORLD_STEP * STEPS_EULER),
            'kernel': 'resident_kernel<128,8>', 'kernel_ms': kern_ms,
            'flops_per_launch': flops_launch,
            'peak_source': 'measured in-bench (FFMA probe kernel, burst); MEASURED_PEAKS.json has no FP32 entry'
        },
        'plain': {
            'value': plain_value, 'unit': METRIC, 'engine': 'fused one-kernel step (resident_kernel, 1 world x 1 step '
                                                          'per launch)',
            'sample': f'{PLAIN_SAMPLE_WORLDS} worlds x {PLAIN_SAMPLE_STEPS} steps, one world and one step per launch, '
                      'L2 flushed before each timed rollout',
            'speedup_batched_vs_plain': value / world_size / plain_value,
            'streamed_sequence': {'value': plain['plain_streamed'], 'kernels_per_world_step': 4,
                                  'speedup_batched_vs_plain': value / world_size / plain['plain_streamed']},
        },
        'adjoint': adjoint,
        'multichannel': multichannel,
        'nd': nd,
        'uneven': uneven,
        'clocks': clocks,
        'gpu_launches': gpu_launches,
        'hbm_peak_gbs_measured': measured_peaks().get('hbm_gbs'),
    }
    return out


def measure_adjoint(dev, worlds=64, steps=256, ckpt=16, reps=3, fp32_peak=None):
    """Differentiation workload: 64 worlds of 128x128 (the single-world model),
    256 steps with checkpoints every 16, MSE of the final state against a
    target made by the forward engine from the same inits at m=0.16, s=0.017;
    gradients with respect to the initial cells, m, s and the ring weights b
    (two rings, so dL/db is not identically zero).  Reports fwd+bwd
    world-steps/s timed with CUDA events around forward + backward, and its
    FP32 roofline: per fwd + bwd world-step the forward step twice (the
    checkpointed forward and the backward's recompute, without statistics)
    plus one reverse step."""
    import torch
    from leniax_gb300 import grad as lgrad
    from leniax_gb300 import helpers, kernels
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in KPARAMS], [SIZE, SIZE], 1, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    cells = torch.from_numpy(make_inputs(worlds, seed=4)).to(dev)
    T = torch.tensor([T_RATE])
    b_t = torch.tensor([1.0, 1.0], device=dev)
    with torch.no_grad():
        kt = lgrad.ring_kernel(R, 1.0, b_t, 'gauss_bump', [1.0], [SIZE, SIZE])[None]
        target = lgrad.rollout(cells, kt, torch.tensor([[[0.16, 0.017]]], device=dev), torch.ones((1, 1, 1),
                                                                                                  device=dev), T,
                               upd, steps, ckpt)
    times = []
    for i in range(reps + 1):
        c0 = cells.clone().requires_grad_(True)
        b = torch.tensor([0.9, 1.0], device=dev, requires_grad=True)
        gf = torch.tensor([[[0.15, 0.015]]], device=dev, requires_grad=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        kr = lgrad.ring_kernel(R, 1.0, b, 'gauss_bump', [1.0], [SIZE, SIZE])[None]
        fin = lgrad.rollout(c0, kr, gf, torch.ones((1, 1, 1), device=dev), T, upd, steps, ckpt)
        loss = ((fin - target)**2).mean()
        loss.backward()
        e1.record()
        torch.cuda.synchronize()
        if i > 0:
            times.append(e0.elapsed_time(e1) / 1e3)
    t = pystats.median(times)
    fpws = 2 * flops_per_world_step(1, 1, P_CELLS, stats=False) + adjoint_flops_per_world_step(P_CELLS)
    achieved = fpws * worlds * steps / t / 1e12
    return {
        'metric': 'fwd+bwd world-steps/s', 'value': worlds * steps / t, 'unit': 'world-steps/s',
        'roofline': {'bound': 'fp32', 'achieved': achieved, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                     'frac': achieved / fp32_peak if fp32_peak else None, 'flops_per_fwd_bwd_world_step': fpws,
                     'note': f'{worlds} worlds take {worlds} of the SMs (one world per SM)'},
        'cell_updates_per_s': worlds * steps * P_CELLS / t, 'seconds': t,
        'config': f'{worlds} worlds x 128x128, {steps} steps, checkpoint every {ckpt}, grads wrt cells0, m, s, b',
        'loss': float(loss.detach()),
        # 256 steps of noise worlds are chaotic: the straight-through gradients of
        # leniax's v1 clip grow without bound over the horizon, so only their
        # finiteness is reported (gradient accuracy is checked at short horizons
        # in tests/test_gpu_adjoint.py)
        'grads_finite': {
            'cells0': bool(torch.isfinite(c0.grad).all()), 'm_s': bool(torch.isfinite(gf.grad).all()),
            'b': bool(torch.isfinite(b.grad).all())
        }
    }


def measure_adjoint_3d(dev, size=48, steps=256, ckpt=16, reps=2):
    """The differentiation workload's 3D variant: one 48x48x48 world (bump
    kernel R=8, gaussian growth m=0.15 s=0.03, dt=0.1, uniform[0,1) central
    16^3 patch), 256 steps with checkpoints every 16, MSE of the final state
    against a target made at m=0.16 s=0.033; gradients with respect to the
    initial cells, the kernel and (m, s) on the general N-D engine (forward
    and adjoint).  fwd+bwd world-steps/s timed with CUDA events."""
    import torch
    from leniax_gb300 import grad as lgrad
    from leniax_gb300 import helpers, kernels
    R, T = 8.0, 10.0
    kp = [dict(KPARAMS[0], gf_params=[0.15, 0.03])]
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size] * 3, 1, R, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    rng = np.random.Generator(np.random.PCG64(5))
    c = np.zeros((1, 1, 1, size, size, size), np.float32)
    lo, p = (size - size // 3) // 2, size // 3
    c[..., lo:lo + p, lo:lo + p, lo:lo + p] = rng.random((p, p, p), dtype=np.float32)
    cells = torch.from_numpy(c).to(dev)
    kr = lgrad.ring_kernel(R, 1.0, torch.tensor([1.0], device=dev), 'gauss_bump', [1.0], [size] * 3)[None]
    with torch.no_grad():
        target = lgrad.rollout(cells, kr, torch.tensor([[[0.16, 0.033]]], device=dev), torch.ones((1, 1, 1), device=dev),
                               torch.tensor([T]), upd, steps, ckpt)
    times = []
    for i in range(reps + 1):
        c0 = cells.clone().requires_grad_(True)
        k0 = kr.clone().requires_grad_(True)
        gf = torch.tensor([[[0.15, 0.03]]], device=dev, requires_grad=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        fin = lgrad.rollout(c0, k0, gf, torch.ones((1, 1, 1), device=dev), torch.tensor([T]), upd, steps, ckpt)
        ((fin - target)**2).mean().backward()
        e1.record()
        torch.cuda.synchronize()
        if i > 0:
            times.append(e0.elapsed_time(e1) / 1e3)
    t = pystats.median(times)
    return {'metric': 'fwd+bwd world-steps/s', 'value': steps / t, 'unit': 'world-steps/s', 'seconds': t,
            'engine': 'nd (forward and adjoint)',
            'config': f'1 world x {size}^3, {steps} steps, checkpoint every {ckpt}, grads wrt cells0, kernel, m, s',
            'grads_finite': bool(torch.isfinite(c0.grad).all() and torch.isfinite(k0.grad).all()
                                 and torch.isfinite(gf.grad).all())}


def _timed(fn, stream, flush, reps):
    """Median CUDA-event time (ms) of fn() over reps runs, L2 flushed before each."""
    import torch
    ts = []
    for _ in range(reps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return pystats.median(ts)


def measure_multichannel(dev, worlds=256, size=256, C=3, per_channel=5, steps=512, reps=2, fp32_peak=None):
    """Multi-channel model on the streamed engine: 256 worlds of 256x256,
    C=3 channels, K=15 kernels (5 per channel, seeded R in [10, 20], 1-3
    rings, m in [0.1, 0.4], s in [0.01, 0.05], target weights normalised per
    channel), dt=0.2, uniform[0,1) 64x64 central patches per channel, 512
    steps with leniax statistics and both stop sets.  Streamed case roofline:
    HBM bytes of the compulsory traffic per Euler step -- every world's state
    in and out (8 C P bytes per world) and each solution's half spectrum in
    once (8 K (P/2+1) bytes; this batch is one solution) -- over the rollout
    time; beside it the FP32 roofline of the algorithmic flops."""
    import torch
    from leniax_gb300 import helpers, kernels, runner, statistics, workloads
    R_world, T_mc = 20.0, 5.0
    kp = workloads.multichannel_params(C, per_channel, seed=0, world_R=R_world)
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], C, R_world, True, dev)
    upd = helpers.build_update_fn(K.shape, mp, 'v1', True)
    stats_fn = statistics.ComputeStatsFn([size, size], R_world, T_mc)
    cells = torch.from_numpy(workloads.multichannel_cells(worlds, C, size, 64, seed=0)[None]).to(dev)
    gf, w, T = mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([T_mc])
    nk = len(kp)
    out = {}

    def run(n_steps):
        out['r'] = runner.run_scan_mem_optimized(None, cells, K[None], gf, w, T, n_steps, R_world, upd, stats_fn,
                                                 engine='streamed', with_box=True)

    run(4)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ms = _timed(lambda: run(steps), torch.cuda.current_stream(dev), flush, reps)
    P = size * size
    cu = worlds * C * P * steps
    n_sols = 1
    bytes_step = 8 * C * P * worlds + 8 * nk * (P // 2 + 1) * n_sols
    achieved = bytes_step * steps / (ms / 1e3) / 1e9
    peak = measured_peaks().get('hbm_gbs')
    flops = flops_per_world_step(C, nk, P) * worlds * steps
    tflops = flops / (ms / 1e3) / 1e12
    sd = out['r'][0]
    return {
        'workload': f'multichannel-{worlds}x{size}x{size}-c{C}k{nk}-{steps}steps', 'engine': 'streamed',
        'metric': METRIC, 'value': cu / (ms / 1e3), 'unit': METRIC, 'ms_per_rollout': ms,
        'ms_per_euler_step': ms / steps, 'mean_N': float(sd['N'].float().mean()),
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak if peak else None,
                     'algorithmic_bytes_per_euler_step': bytes_step,
                     'note': 'compulsory traffic over the whole step; peak = measured copy bandwidth'},
        'roofline_fp32': {'bound': 'fp32', 'achieved': tflops, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                          'frac': tflops / fp32_peak if fp32_peak else None,
                          'flops_per_world_step': flops_per_world_step(C, nk, P)},
        'l2': 'flushed between timed rollouts (256 MB write)',
    }


def measure_nd(dev, worlds=64, size=48, steps=64, reps=2, fp32_peak=None):
    """The general N-D engine on 3D worlds no specialised engine serves: 64
    worlds of 48x48x48 (bump kernel R=8, gaussian growth m=0.15 s=0.03,
    dt=0.1, uniform[0,1) central 16^3 patches), 64 steps with leniax
    statistics and both stop sets; FP32 roofline of the algorithmic flops."""
    import torch
    from leniax_gb300 import helpers, kernels, runner, statistics
    R_nd = 8.0
    kp = [dict(KPARAMS[0], gf_params=[0.15, 0.03])]
    K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size] * 3, 1, R_nd, True, dev)
    upd = helpers.build_update_fn(K.shape, mp)
    stats_fn = statistics.ComputeStatsFn([size] * 3, R_nd, T_RATE)
    rng = np.random.Generator(np.random.PCG64(5))
    c = np.zeros((1, worlds, 1, size, size, size), np.float32)
    lo, p = (size - size // 3) // 2, size // 3
    c[..., lo:lo + p, lo:lo + p, lo:lo + p] = rng.random((worlds, 1, p, p, p), dtype=np.float32)
    cells = torch.from_numpy(c).to(dev)
    gf, w, T = mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([T_RATE])

    def run(n_steps):
        return runner.run_scan_mem_optimized(None, cells, K[None], gf, w, T, n_steps, R_nd, upd, stats_fn,
                                             with_box=True)

    run(4)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ms = _timed(lambda: run(steps), torch.cuda.current_stream(dev), flush, reps)
    P = size**3
    flops = flops_per_world_step(1, 1, P) * worlds * steps
    tflops = flops / (ms / 1e3) / 1e12
    return {
        'workload': f'nd-{worlds}x{size}x{size}x{size}-c1k1-{steps}steps', 'engine': 'nd', 'metric': METRIC,
        'value': worlds * P * steps / (ms / 1e3), 'unit': METRIC, 'ms_per_rollout': ms,
        'ms_per_euler_step': ms / steps,
        'roofline_fp32': {'bound': 'fp32', 'achieved': tflops, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                          'frac': tflops / fp32_peak if fp32_peak else None,
                          'flops_per_world_step': flops_per_world_step(1, 1, P)},
        'l2': 'flushed between timed rollouts (256 MB write)',
    }


def measure_uneven(dev, steps=256, reps=3, fp32_peak=None):
    """Uneven search batch in one persistent launch, replayed from a CUDA
    graph: 4096 C=K=1 worlds (2048 of 64x64, 1229 of 128x128, 614 of
    256x256, 205 of 64x64x64), per-world R in [5, 26], m in [0.1, 0.35], s in
    [0.01, 0.05], dt in {0.05, 0.1, 0.2}, uniform[0,1) central patches of side
    size/3, 256 steps, statistics and both stop sets per world.  Settings from
    the autotuner.  Beside it: the same classes launched one class after the
    other (one shape per launch, as a shape-specialised vmap batches them)."""
    import torch
    from leniax_gb300 import autotune
    from leniax_gb300 import batch as lbatch
    from leniax_gb300 import workloads
    classes = workloads.build_classes(device=dev)
    t0 = time.perf_counter()
    settings = autotune.tuned_settings(classes, steps)
    tune_s = time.perf_counter() - t0
    b = lbatch.UnevenBatch(classes, steps, **settings).capture()
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    b.run()
    torch.cuda.synchronize()
    ms = _timed(b.run, stream, flush, reps)
    per_class = [lbatch.UnevenBatch([c], steps, line_group=settings.get('line_group', 4)).capture() for c in classes]
    for pc in per_class:
        pc.run()
    torch.cuda.synchronize()

    def seq():
        for pc in per_class:
            pc.run()

    ms_seq = _timed(seq, stream, flush, max(1, reps - 1))
    res = b.results()
    n_alive = sum(float(r['stats']['N_box'].sum()) for r in res) / sum(c.n for c in classes)
    flops = sum(c.n * flops_per_world_step(1, 1, int(np.prod(c.world))) for c in classes) * steps
    tflops = flops / (ms / 1e3) / 1e12
    return {
        'workload': 'uneven-4096-worlds-64sq-128sq-256sq-64cube-256steps', 'metric': METRIC,
        'value': b.cells_per_run / (ms / 1e3), 'unit': METRIC, 'ms_per_rollout': ms,
        'roofline': {'bound': 'fp32', 'achieved': tflops, 'peak': fp32_peak, 'unit': 'TFLOP/s',
                     'frac': tflops / fp32_peak if fp32_peak else None, 'flops_per_rollout': flops},
        'classes': [{'world': list(c.world), 'worlds': c.n} for c in classes],
        'settings': settings, 'autotune_seconds': tune_s, 'graph': True,
        'one_class_per_launch': {'value': b.cells_per_run / (ms_seq / 1e3), 'ms_per_rollout': ms_seq},
        'mean_stop_step_box_set': n_alive, 'l2': 'flushed between timed rollouts (256 MB write)',
    }


def profile_case(args):
    """Small cases for ncu captures: one warm-up and one timed run of the
    named workload, nothing else.
      resident     : the search batch (--profile-worlds worlds x 128x128 x --profile-steps steps)
      multichannel : the multi-channel model on the streamed engine
                     (--profile-worlds worlds x 256x256, C=3, K=15, --profile-steps steps)
      uneven256 / uneven3d : --profile-worlds worlds of 256x256 / 64x64x64 in one uneven-batch launch
                     (--profile-steps steps)
      adjoint      : the differentiation workload (forward + backward) on --profile-worlds worlds of
                     128x128 over --profile-steps steps, checkpoints every 16
      nd48         : --profile-worlds worlds of 48x48x48 (bump kernel R=8, gaussian growth) on the
                     general N-D engine, --profile-steps steps with statistics
      adjoint3d    : the differentiation workload's 3D variant (one 48x48x48 world, forward + backward
                     on the N-D engine) over --profile-steps steps, checkpoints every 16"""
    import torch
    from leniax_gb300 import helpers, kernels, runner, statistics
    dev = torch.device('cuda', 0)
    name, nw, ns = args.profile_case, args.profile_worlds, args.profile_steps
    if name == 'resident':
        K, mp = kernels.get_kernels_and_mapping([dict(p) for p in KPARAMS], [SIZE, SIZE], 1, R, True, dev)
        upd = helpers.build_update_fn(K.shape, mp)
        stats_fn = statistics.ComputeStatsFn([SIZE, SIZE], R, T_RATE)
        cells = torch.from_numpy(make_inputs(nw, seed=1)).to(dev)
        gf, w, Tt = mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([T_RATE])
        for _ in range(2):
            sd, fin = runner.run_scan_mem_optimized(None, cells, K[None], gf, w, Tt, ns, R, upd, stats_fn,
                                                    with_box=True, with_centroid=True)
        info = {'mean_N_box': float(sd['N_box'].mean())}
    elif name == 'multichannel':
        from leniax_gb300 import workloads
        C, size, Rw, Tm = 3, 256, 20.0, 5.0
        kp = workloads.multichannel_params(C, 5, seed=0, world_R=Rw)
        K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size, size], C, Rw, True, dev)
        upd = helpers.build_update_fn(K.shape, mp, 'v1', True)
        stats_fn = statistics.ComputeStatsFn([size, size], Rw, Tm)
        cells = torch.from_numpy(workloads.multichannel_cells(nw, C, size, 64, seed=0)[None]).to(dev)
        gf, w, Tt = mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([Tm])
        for _ in range(2):
            sd, fin = runner.run_scan_mem_optimized(None, cells, K[None], gf, w, Tt, ns, Rw, upd, stats_fn,
                                                    engine='streamed', with_box=True)
        info = {'mean_N': float(sd['N'].float().mean())}
    elif name == 'adjoint':
        r = measure_adjoint(dev, worlds=nw, steps=ns, reps=1)
        info = {'fwd_bwd_world_steps_per_s': r['value']}
    elif name == 'adjoint3d':
        r = measure_adjoint_3d(dev, steps=ns, reps=1)
        info = {'fwd_bwd_world_steps_per_s': r['value']}
    elif name == 'nd48':
        size, Rn = 48, 8.0
        kp = [dict(KPARAMS[0], gf_params=[0.15, 0.03])]
        K, mp = kernels.get_kernels_and_mapping([dict(p) for p in kp], [size] * 3, 1, Rn, True, dev)
        upd = helpers.build_update_fn(K.shape, mp)
        stats_fn = statistics.ComputeStatsFn([size] * 3, Rn, T_RATE)
        rng = np.random.Generator(np.random.PCG64(5))
        c = np.zeros((1, nw, 1, size, size, size), np.float32)
        lo, p = (size - size // 3) // 2, size // 3
        c[..., lo:lo + p, lo:lo + p, lo:lo + p] = rng.random((nw, 1, p, p, p), dtype=np.float32)
        cells = torch.from_numpy(c).to(dev)
        gf, w, Tt = mp.get_gf_params(dev)[None], mp.get_kernels_weight_per_channel(dev)[None], torch.tensor([T_RATE])
        for _ in range(2):
            sd, fin = runner.run_scan_mem_optimized(None, cells, K[None], gf, w, Tt, ns, Rn, upd, stats_fn,
                                                    with_box=True)
        info = {'mean_N_box': float(sd['N_box'].mean())}
    else:
        from leniax_gb300 import batch as lbatch
        from leniax_gb300 import workloads
        world = (256, 256) if name == 'uneven256' else (64, 64, 64)
        b = lbatch.UnevenBatch(workloads.build_classes(mix=[(world, nw)], device=dev), ns)
        for _ in range(2):
            b.run()
        info = {'mean_N_box': float(b.results()[0]['stats']['N_box'].mean())}
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': name, 'worlds': nw, 'steps': ns, **info}))


def run_reference(args, budget_s=90.0):
    """Reference arm: the reference's CPU algorithm for this path (leniax's JAX
    is not installable here, so its numpy restatement), all host threads.
    One step is one bounded sample of the workload (CPU_SAMPLE_WORLDS worlds
    from their initial states, the same number of Euler steps each time),
    sized from a short calibration so that the ``warmup + steps`` samples take
    about ``budget_s`` seconds; ``steps`` samples are timed."""
    smp = _OracleSample()
    cal_steps = 8
    smp.run(2)
    per_step = smp.run(cal_steps) / cal_steps
    n_samples = max(1, args.warmup + args.steps)
    euler = int(min(CPU_SAMPLE_STEPS, max(16, budget_s / n_samples / per_step)))
    for _ in range(args.warmup):
        smp.run(euler)
    times = [smp.run(euler) for _ in range(max(1, args.steps))]
    total = sum(times)
    value = CPU_SAMPLE_WORLDS * P_CELLS * euler * len(times) / total
    cb = {'value': value, 'unit': METRIC, 'cores': smp.cores, 'kind': 'port',
          'sample': smp.describe(euler, total / len(times)) + ' per step'}
    return {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': METRIC, 'n_gpus': args.gpus,
        'steps': len(times), 'warmup': args.warmup, 'ms_per_step': 1e3 * total / len(times),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic (PCG64 seeded uniform patches)',
        'config': {'workload': WORKLOAD, 'parallelism': 'host cores',
                   'step': f'{CPU_SAMPLE_WORLDS} worlds x {euler} Euler steps of the workload'},
        'cpu_baseline': cb,
        'e2e': {'value': value, 'unit': METRIC, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--profile-case', nargs='?', const='resident', default=None,
                    choices=['resident', 'multichannel', 'uneven256', 'uneven3d', 'adjoint', 'nd48', 'adjoint3d'],
                    help='profiling case for ncu: one warm-up and one rollout of --profile-worlds worlds x '
                         '--profile-steps Euler steps of the named workload, nothing else')
    ap.add_argument('--profile-worlds', type=int, default=2048)
    ap.add_argument('--profile-steps', type=int, default=16)
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args)
        return
    world_size = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if args.impl == 'reference':
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world_size > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', 0)))
        torch.distributed.init_process_group('nccl')
    out = run_ours(args, rank, world_size)
    if rank == 0:
        out['cpu_baseline'] = cpu_baseline()
        print(json.dumps(out))
    if world_size > 1:
        import torch
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
