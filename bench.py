#!/usr/bin/env python3
"""Benchmark of the tensor-train ALS hot path on one GB300.

Workload: SLE ALS on the coupled Laplacian (d=32 sites, mode size n=8,
operator rank 4, right-hand side rank 8, solution rank 32, 4 sweeps, seeded
inputs).  A *step* is one full solve.

* ``value``: solves/s of the mixed-precision engine (FP32 Krylov inner solves,
  FP64 refinement residual, FP64 stacks and QR) with the inputs resident in HBM,
  timed with CUDA events on the engine's stream, L2 flushed between steps.
* ``e2e``: the same solve through the C ABI with host buffers (host->device
  copies of the three trains and the device->host copy of the solution inside
  the timed region), wall clock.
* ``plain_fp64``: the plain FP64 engine on the same inputs (the drop-in
  baseline the mixed path is compared with).
* ``cpu_baseline``: the CPU oracle (a NumPy restatement of the reference's
  dense-LU ALS) on a bounded sample of the same workload, extrapolated.

``--impl reference`` times only that CPU restatement (the reference itself is
pure Python and is not shipped to the GPU host).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'solves/s at rel. residual≤1e-8, mixed vs plain FP64 on GB300; p50/p99 latency'
UNIT = 'solves/s'
WORKLOAD = dict(d=32, n=8, rhs_rank=8, x_rank=32, repeats=4)
WORKLOAD_NAME = 'coupled-Laplacian SLE ALS, d=32 n=8 op_rank=4 rhs_rank=8 x_rank=32, 4 sweeps'
MIXED_TOL = 1e-10


def dist_env():
    return int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1')), \
        int(os.environ.get('LOCAL_RANK', '0'))


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's dense-LU ALS on a bounded sample
# ---------------------------------------------------------------------------

def site_sizes(w):
    """N = r_i n r_{i+1} of every local solve of the run (rank rule of the
    reference's economic QR/RQ)."""
    d, n = w.meta['d'], w.meta['n']
    r = [1] + [w.meta['x_rank']] * (d - 1) + [1]
    for i in range(d - 1, 0, -1):
        r[i] = min(r[i], n * r[i + 1])
    sizes = []
    for _ in range(w.repeats):
        for i in range(d - 1):
            sizes.append(r[i] * n * r[i + 1])
            r[i + 1] = min(r[i] * n, r[i + 1])
        for i in range(d - 1, -1, -1):
            sizes.append(r[i] * n * r[i + 1])
            if i > 0:
                r[i] = min(r[i], n * r[i + 1])
    return sizes


def cpu_sample(w, nsites=2):
    """Time ``nsites`` full-size local steps (stack update, dense local matrix,
    LU solve, QR) of the oracle and extrapolate to the whole run by N^3."""
    from oracle import tt_oracle as O
    d = len(w.op)
    cores = O.ortho_right(w.x0)
    b = w.rhs
    sr_op, sr_b = [None] * d, [None] * d
    sr_op[d - 1], sr_b[d - 1] = np.ones((1, 1, 1)), np.ones((1, 1))
    for i in range(d - 2, -1, -1):
        x = cores[i + 1][:, :, 0, :]
        sr_op[i] = O.stack_right_op(sr_op[i + 1], x, w.op[i + 1])
        sr_b[i] = O.stack_right_vec(sr_b[i + 1], x, b[i + 1][:, :, 0, :])
    L, Lb = np.ones((1, 1, 1)), np.ones((1, 1))
    times, ns = [], []
    ranks = [c.shape[0] for c in cores] + [1]
    for i in range(d - 1):
        t0 = time.perf_counter()
        if i > 0:
            x = cores[i - 1][:, :, 0, :]
            L = O.stack_left_op(L, x, w.op[i - 1])
            Lb = O.stack_left_vec(Lb, x, b[i - 1][:, :, 0, :])
        M = O.micro_matrix(L, w.op[i], sr_op[i])
        f = O.micro_vec(Lb, b[i][:, :, 0, :], sr_b[i])
        y = np.linalg.solve(M, f)
        a, n, s = ranks[i], w.op[i].shape[1], ranks[i + 1]
        q, _ = np.linalg.qr(y.reshape(a * n, s))
        ranks[i + 1] = q.shape[1]
        cores[i] = q.reshape(a, n, 1, q.shape[1])
        dt = time.perf_counter() - t0
        N = a * n * s
        if N == max(site_sizes(w)):
            times.append(dt)
            ns.append(N)
            if len(times) >= nsites:
                break
    t_big = float(np.median(times))
    nmax = ns[0]
    est = sum(t_big * (N / nmax) ** 3 for N in site_sizes(w))
    return est, len(times), nmax


def cpu_threads():
    for k in ('OPENBLAS_NUM_THREADS', 'OMP_NUM_THREADS'):
        if os.environ.get(k):
            return int(os.environ[k])
    return os.cpu_count() or 1


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from scikit_tt_gb300 import workloads as wl
    w = wl.coupled_sle(**WORKLOAD)
    for _ in range(args.warmup):
        cpu_sample(w, nsites=1)
    vals = []
    for _ in range(args.steps):
        est, k, nmax = cpu_sample(w, nsites=1)
        vals.append(1.0 / est)
    v = float(np.median(vals))
    sample = f'{1} local step(s) at N={nmax} per step (stack, dense N x N matrix, LU solve, QR), ' \
             f'extrapolated by N^3 to the {len(site_sizes(w))} local solves of one run'
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': args.gpus, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1e3 / v, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
        'config': {'workload': WORKLOAD_NAME, 'precision': 'fp64 dense LU (NumPy/SciPy restatement)'},
        'cpu_baseline': {'value': v, 'unit': UNIT, 'cores': cpu_threads(), 'kind': 'port', 'sample': sample},
        'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = 'index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,' \
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,' \
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap'

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            p = [x.strip() for x in ln.split(',')]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, v in zip(names, p[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(k)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled'], 'samples': 0}
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': float(max(mx)), 'reasons': sorted(reasons),
                'samples': len(sm)}


def main_gpu(args):
    import torch
    from scikit_tt_gb300 import _lib
    from scikit_tt_gb300 import workloads as wl

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    torch.cuda.set_device(local)
    os.environ['TTALS_DEVICE'] = str(local)
    dev = torch.device('cuda', local)
    lib = _lib.load()
    ctx = _lib.context()
    stream = torch.cuda.current_stream(dev)
    _lib.check(lib.ttals_set_stream(ctx, _lib.C.c_void_p(stream.cuda_stream)))

    # each rank solves its own replica (independent seeded instance)
    w = wl.coupled_sle(seed=rank, **WORKLOAD)
    packs = [_lib.Packed(t) for t in (w.op, w.x0, w.rhs)]
    dev_bufs = [torch.from_numpy(p.data).to(dev) for p in packs]
    dev_descs = []
    for p, b in zip(packs, dev_bufs):
        dev_descs.append(_lib.TTDesc(p.order, _lib.i64ptr(p.row), _lib.i64ptr(p.col), _lib.i64ptr(p.ranks),
                                     _lib.C.cast(b.data_ptr(), _lib.C.POINTER(_lib.C.c_double)), 1))
    dims = np.array([c.shape[1] for c in w.op], dtype=np.int64)
    out_ranks = np.zeros(len(w.op) + 1, dtype=np.int64)
    _lib.check(lib.ttals_als_ranks(len(w.op), _lib.i64ptr(dims), _lib.i64ptr(packs[1].ranks), _lib.i64ptr(out_ranks)))
    out_total = int(sum(out_ranks[i] * dims[i] * out_ranks[i + 1] for i in range(len(w.op))))
    out_dev = torch.empty(out_total, dtype=torch.float64, device=dev)
    out_host = np.empty(out_total, dtype=np.float64)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def solve_dev(prec, tol, stats=None):
        st = stats if stats is not None else _lib.Stats()
        _lib.check(lib.ttals_sle_als(ctx, dev_descs[0], dev_descs[1], dev_descs[2], w.repeats, 0, prec, tol,
                                     _lib.C.cast(out_dev.data_ptr(), _lib.C.POINTER(_lib.C.c_double)), 1,
                                     _lib.i64ptr(out_ranks), st))
        return st

    def solve_host(prec, tol):
        st = _lib.Stats()
        _lib.check(lib.ttals_sle_als(ctx, packs[0].desc, packs[1].desc, packs[2].desc, w.repeats, 0, prec, tol,
                                     _lib.dptr(out_host), 0, _lib.i64ptr(out_ranks), st))
        return st

    def timed(prec, tol, steps, warmup):
        for _ in range(warmup):
            solve_dev(prec, tol)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        launches, stats = 0, []
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            st = solve_dev(prec, tol)
            ev[k][1].record(stream)
            launches += st.kernel_launches
            stats.append(st.as_dict())
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in ev]
        return ms, launches, stats

    # arithmetic peaks of this device (FMA chains), for the roofline fractions
    p64, p32 = _lib.C.c_double(0), _lib.C.c_double(0)
    _lib.check(lib.ttals_measure_peaks(ctx, _lib.C.byref(p64), _lib.C.byref(p32)))

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms_mixed, launches, st_mixed = timed(_lib.PREC_MIXED, MIXED_TOL, args.steps, args.warmup)
    torch.cuda.synchronize()
    total_ms = float(np.sum(ms_mixed))
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms / 1e3)
    mixed_sol = out_dev.cpu().numpy().copy()

    # plain FP64 drop-in on the same inputs
    plain_steps = max(1, min(args.steps, 3))
    ms_plain, _, st_plain = timed(_lib.PREC_FP64, 0.0, plain_steps, 1)
    plain_sol = out_dev.cpu().numpy().copy()
    plain_value = 1e3 / float(np.mean(ms_plain))

    # agreement of the mixed and plain solutions (device TT norm)
    from scikit_tt_gb300.tensor_train import TT
    rk = [int(r) for r in out_ranks]
    tm = TT(_lib.unpack(mixed_sol, dims, [1] * len(dims), rk))
    tp = TT(_lib.unpack(plain_sol, dims, [1] * len(dims), rk))
    mixed_vs_plain = (tm - tp).norm() / tp.norm()

    # end to end through the C ABI with host buffers
    e2e_ms = []
    for _ in range(2):
        solve_host(_lib.PREC_MIXED, MIXED_TOL)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        solve_host(_lib.PREC_MIXED, MIXED_TOL)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    h2d = sum(p.data.nbytes for p in packs)
    d2h = out_host.nbytes + 8 * len(out_ranks)

    # roofline of the local-solve kernel: profiled pass, live CUDA events
    _lib.check(lib.ttals_set_profiling(ctx, 1))
    prof = solve_dev(_lib.PREC_MIXED, MIXED_TOL)
    prof_plain = solve_dev(_lib.PREC_FP64, 0.0)
    _lib.check(lib.ttals_set_profiling(ctx, 0))
    torch.cuda.synchronize()
    per_launch_s = prof.solver_ms / max(prof.solver_launches, 1) / 1e3
    ach64 = prof.solver_flops64 / max(prof.solver_launches, 1) / per_launch_s / 1e9
    ach32 = prof.solver_flops32 / max(prof.solver_launches, 1) / per_launch_s / 1e9
    plain_per_launch_s = prof_plain.solver_ms / max(prof_plain.solver_launches, 1) / 1e3
    plain_ach64 = prof_plain.solver_flops64 / max(prof_plain.solver_launches, 1) / plain_per_launch_s / 1e9
    traffic = None
    tf = os.path.join(ROOT, 'profiles', 'traffic.json')
    if os.path.exists(tf):
        traffic = json.load(open(tf)).get('gmres_ir_kernel<float>')

    if rank != 0:
        return
    cpu_est, nsamp, nmax = cpu_sample(w, nsites=2)
    lat = np.array(ms_mixed)
    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': total_ms / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 Krylov + f64 refinement/stacks/QR',
        'data': 'synthetic (seeded N(0,1) trains)',
        'config': {'workload': WORKLOAD_NAME, 'precision': 'mixed', 'local_tol': MIXED_TOL, 'batch': 1,
                   'l2': 'flushed between steps (256 MiB write)', 'parallelism': f'replicas x{world}'},
        'latency_ms': {'p50': float(np.percentile(lat, 50)), 'p99': float(np.percentile(lat, 99)),
                       'mean': float(lat.mean())},
        'plain_fp64': {'value': plain_value, 'unit': UNIT, 'ms_per_solve': float(np.mean(ms_plain)),
                       'max_local_residual': st_plain[-1]['max_local_residual'],
                       'solver_achieved_fp64_gflops': plain_ach64},
        'mixed_over_plain': value / world / plain_value,
        'mixed_vs_plain_rel_diff': mixed_vs_plain,
        'max_local_residual': max(s['max_local_residual'] for s in st_mixed),
        'e2e': {'value': 1e3 / float(np.mean(e2e_ms)), 'unit': UNIT, 'h2d_bytes_per_step': int(h2d),
                'd2h_bytes_per_step': int(d2h), 'p50_ms': float(np.percentile(e2e_ms, 50)),
                'p99_ms': float(np.percentile(e2e_ms, 99))},
        'gpu_launches': int(launches),
        'roofline': {'kernel': 'gmres_ir_kernel<float> (local solve)', 'bound': 'fp64',
                     'achieved': ach64, 'peak': p64.value, 'unit': 'GFLOP/s', 'frac': ach64 / p64.value,
                     'traffic': traffic, 'peak_source': 'FP64 FMA-chain microbenchmark run in this process',
                     'achieved_fp32_gflops': ach32, 'fp32_peak_gflops': p32.value,
                     'avg_launch_ms': per_launch_s * 1e3,
                     'share_of_step': prof.solver_ms / max(prof.device_ms, 1e-9)},
        'cpu_baseline': {'value': 1.0 / cpu_est, 'unit': UNIT, 'cores': cpu_threads(), 'kind': 'port',
                         'sample': f'{nsamp} oracle local steps at N={nmax} (stack, dense matrix, LU, QR), '
                                   f'extrapolated by N^3 to all local solves of one run'},
        'clocks': clk.summary(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    args = ap.parse_args()
    if args.impl == 'reference':
        run_reference(args)
    else:
        main_gpu(args)


if __name__ == '__main__':
    main()
