"""Benchmark of the jax-cfd hot path on GB300 (one JSON line on stdout).

Workload (the configuration the headline metric is quoted on): the
staggered-grid semi_implicit_navier_stokes step (Van Leer advection, explicit
diffusion, Kolmogorov sin(4y) + linear drag -0.1 forcing, solve_fast_diag
projection, forward Euler) on a 2048 x 2048 periodic [0, 2pi]^2 float32 grid,
nu = 1e-3, rho = 1, dt = stable_time_step(2, 0.5) = 7.6699e-4, from a seeded
filtered random velocity field with max speed 2 (synthetic: no dataset exists
for this path).  One bench "step" is one ``funcutils.repeated(step, chunk)``
call, i.e. `chunk` (default 200) FVM time steps; the default 10 timed steps
are the 2000 steps of the 2048^2 scale-up configuration.

Timing: CUDA events around each chunk on the launching stream, the L2 flushed
(a 256 MiB write) between chunks, a barrier + synchronize on both sides of the
timed loop, max over ranks.  `value` = grid cells x time steps / second with
the state resident in HBM; `e2e` is the same metric through the public API
with the velocity copied from pinned host memory before, and back after,
every chunk.  `roofline` uses per-kernel CUDA-event durations from a second
pass over the same workload and the HBM bandwidth in MEASURED_PEAKS.json.

`--impl reference` times the reference algorithm on the host CPU (the NumPy
restatement of jax-cfd's step; JAX cannot be installed here) on a bounded
sample of the same workload: one 2048^2 trajectory per host core, in spawned
processes timed together.

Multi-GPU: replicas only (each rank advances its own trajectory; no
collective on the data path); value sums the ranks' cell-steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)

N = 2048
VISCOSITY = 1e-3
MAX_VELOCITY = 2.0
CFL = 0.5
DOMAIN = ((0, 2 * np.pi), (0, 2 * np.pi))
# Algorithmic HBM bytes per cell and FVM step (float32): explicit stencil reads
# u*, v*, q and writes u*, v* (20); divergence + row rFFT reads u*, v*, writes
# the packed spectrum (12); column pass reads/writes the spectrum (8); row
# irFFT reads/writes it (8).
# The headline workload, named alike on both arms (the metric is cell-steps/s;
# the arms differ only in how many time steps one bench step holds).
def fvm_workload(n: int) -> str:
  return (f'semi_implicit_navier_stokes {n}x{n} float32, Van Leer, nu=1e-3, '
          'Kolmogorov k=4 + drag 0.1, forward Euler, seeded filtered initial field')


FVM_BYTES_PER_CELL = {'explicit': 20, 'div_rfft': 12, 'col_pinv': 8, 'irfft': 8,
                      'project_out': 20}
FVM_STEP_BYTES_PER_CELL = 48
# Spectral stage (per cell of the N x N grid): row pass reads 4 complex
# half-spectrum fields (16) and writes one (4); column update reads the
# advection spectrum, state and h (12) and writes state and h (8); column prep
# reads the state (4) and writes 4 fields (16); the fused column stage (update
# and the next stage's prep in one pass) is both without the prep's state
# read (36).
SPEC_BYTES_PER_CELL = {'row': 20, 'col_update': 20, 'col_prep': 20, 'col_stage': 36}
SPEC_STEP_BYTES_PER_CELL = 300


def _peaks():
  path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
  try:
    with open(path) as f:
      d = json.load(f)
    return float(d['hbm_gbs']), 'measured'
  except Exception:  # pylint: disable=broad-except
    return 6800.0, 'fallback'


def spectral_launches_per_time_step(chunk: int) -> dict:
  """Launches of each spectral kernel per time step in a chunk of `chunk`
  steps: five row passes and five column stages per step, of which the last
  of the chunk is the plain update; the prep runs once per chunk."""
  return {'row': 5.0, 'col_stage': 5.0 - 1.0 / chunk, 'col_update': 1.0 / chunk,
          'col_prep': 1.0 / chunk}


def spectral_dominant_kernel(kernel_ms: dict, chunk: int) -> str:
  """The spectral kernel with the most device time per time step."""
  per_step = spectral_launches_per_time_step(chunk)
  return max(per_step, key=lambda k: kernel_ms[k] * per_step[k])


def _traffic_table():
  path = os.path.join(ROOT, 'profiles', 'dram_traffic.json')
  try:
    with open(path) as f:
      return json.load(f)
  except Exception:  # pylint: disable=broad-except
    return {}


class ClockSampler:
  """Samples nvidia-smi clocks and throttle reasons while running."""
  QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
           'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
           'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

  def __init__(self, index: int):
    self.index = index
    self.proc = None
    self.lines = []
    self._t = None

  def __enter__(self):
    try:
      self.proc = subprocess.Popen(
          ['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.QUERY}',
           '--format=csv,noheader,nounits', '-lms', '200'],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self._t = threading.Thread(target=self._read, daemon=True)
      self._t.start()
    except Exception:  # pylint: disable=broad-except
      self.proc = None
    return self

  def _read(self):
    for line in self.proc.stdout:
      self.lines.append(line.strip())

  def __exit__(self, *exc):
    if self.proc is not None:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except Exception:  # pylint: disable=broad-except
        self.proc.kill()
      if self._t is not None:
        self._t.join(timeout=2)

  def summary(self):
    sm, smax, reasons = [], [], set()
    names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
    for line in self.lines:
      parts = [p.strip() for p in line.split(',')]
      if len(parts) < 9:
        continue
      try:
        sm.append(float(parts[1]))
        smax.append(float(parts[2]))
      except ValueError:
        continue
      for name, val in zip(names, parts[5:9]):
        if val.lower().startswith('active'):
          reasons.add(name)
    if not sm:
      return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unsampled'], 'samples': 0}
    return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': max(smax),
            'reasons': sorted(reasons), 'samples': len(sm)}


def _dist():
  world = int(os.environ.get('WORLD_SIZE', '1'))
  rank = int(os.environ.get('RANK', '0'))
  local = int(os.environ.get('LOCAL_RANK', '0'))
  return world, rank, local


def _json_line(obj):
  print(json.dumps(obj), flush=True)


def max_over_ranks(x: float) -> float:
  """Max of a per-rank float over the process group (identity without one).

  Ranks are independent replicas, so this is the only cross-rank operation:
  the slowest rank's timed region defines the job's time."""
  import torch  # pylint: disable=import-outside-toplevel
  import torch.distributed as dist  # pylint: disable=import-outside-toplevel
  if not (dist.is_available() and dist.is_initialized()):
    return float(x)
  dev = (torch.device('cuda', torch.cuda.current_device())
         if dist.get_backend() == 'nccl' else torch.device('cpu'))
  t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


# ---------------------------------------------------------------------------
# Reference arm: the jax-cfd algorithm on the host CPU.
# ---------------------------------------------------------------------------
def _cpu_step(n: int, seed: int):
  """The NumPy restatement of the reference step at n x n from the seeded
  filtered initial field of the GPU arm's workload (max speed 2, peak
  wavenumber 4)."""
  from oracle import fvm as ofvm  # pylint: disable=import-outside-toplevel
  from oracle import initial_conditions as oic  # pylint: disable=import-outside-toplevel
  og = ofvm.Grid.make((n, n), domain=DOMAIN)
  v = oic.filtered_velocity_field(seed, og, MAX_VELOCITY, 4)
  dt = ofvm.stable_time_step(MAX_VELOCITY, CFL, VISCOSITY, og)
  step = ofvm.semi_implicit_navier_stokes(
      1.0, VISCOSITY, dt, og, forcing=ofvm.simple_turbulence_forcing(og, 1, 4, -0.1))
  return step, v


def _cpu_worker(index: int, steps: int, warmup: int, n: int, barrier, results):
  """One host process of the CPU sample: warm up, wait for every process,
  then time `steps` steps (monotonic clock, comparable across processes)."""
  step, v = _cpu_step(n, index)
  for _ in range(warmup):
    v = step(v)
  barrier.wait()
  t0 = time.perf_counter()
  for _ in range(steps):
    v = step(v)
  results.put((t0, time.perf_counter()))


def _cpu_sample(steps: int, warmup: int, n: int = N, procs: int = 0):
  """Times the NumPy restatement of the reference step on a bounded sample:
  `procs` host processes (default: one per host core, started with spawn),
  each advancing its own n x n trajectory by `steps` steps after `warmup`;
  returns (cell-steps/s over all processes, seconds of the timed region,
  processes).  The restatement is single-threaded, so one trajectory per core
  is how it uses every core."""
  import multiprocessing  # pylint: disable=import-outside-toplevel
  procs = procs or os.cpu_count() or 1
  ctx = multiprocessing.get_context('spawn')
  barrier = ctx.Barrier(procs)
  results = ctx.Queue()
  workers = [ctx.Process(target=_cpu_worker, args=(i, steps, warmup, n, barrier, results))
             for i in range(procs)]
  for w in workers:
    w.start()
  spans = [results.get() for _ in range(procs)]
  for w in workers:
    w.join()
  secs = max(t1 for _, t1 in spans) - min(t0 for t0, _ in spans)
  return procs * n * n * steps / secs, secs, procs


def run_reference(args):
  world, rank, _ = _dist()
  if rank != 0:
    return
  k = max(1, args.steps)
  w = max(0, args.warmup)
  # Each reference "step" is one FVM time step of the 2048^2 workload (a
  # bounded sample: the full 2000-step run would take about an hour on CPU).
  value, secs, threads = _cpu_sample(k, w)
  sample = (f'{threads} host processes (one per core), each {k} FVM steps of its own '
            f'{N}x{N} trajectory after {w} warm-up steps ({secs:.1f} s)')
  _json_line({
      'metric': 'FVM cell-steps/s at 2048^2', 'value': value, 'unit': 'cell-steps/s',
      'impl': 'reference', 'n_gpus': world, 'steps': k, 'warmup': w,
      'ms_per_step': 1000.0 * secs / k, 'higher_is_better': True, 'scaling': 'weak',
      'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
      'config': {'workload': fvm_workload(N), 'grid': [N, N], 'parallelism': 'host',
                 'implementation': 'NumPy restatement of the reference on the host CPU, one '
                                   'time step per bench step (a bounded sample)'},
      'cpu_baseline': {'value': value, 'unit': 'cell-steps/s', 'cores': threads,
                       'kind': 'port', 'sample': sample},
      'e2e': {'value': value, 'unit': 'cell-steps/s', 'h2d_bytes_per_step': 0,
              'd2h_bytes_per_step': 0},
  })


# ---------------------------------------------------------------------------
# GB300 arm.
# ---------------------------------------------------------------------------
def ensemble_draws(count: int, seed: int = 2024):
  """Members of the ragged FVM ensemble: grid N uniform in {64..1024},
  viscosity log-uniform in [1e-4, 1e-2], forcing wavenumber in {2, 4, 8}, max
  initial speed uniform in [1, 4], initial-condition seed 1000 + i.  dt is
  stable_time_step(vmax, 0.5, nu) where the reference accepts it, else the
  diffusive limit h^2 / (4 nu) (the reference raises for those draws)."""
  rng = np.random.default_rng(seed)
  out = []
  for i in range(count):
    n = int(rng.choice([64, 128, 256, 512, 1024]))
    nu = float(10 ** rng.uniform(-4, -2))
    k = int(rng.choice([2, 4, 8]))
    vmax = float(rng.uniform(1, 4))
    h = 2 * np.pi / n
    dt = min(CFL * h / vmax, h * h / (4 * nu))
    out.append(dict(n=n, nu=nu, k=k, vmax=vmax, dt=dt, seed=1000 + i))
  return out


def run_ensemble(dev, args, flush):
  """Ragged ensemble (batched launches per grid shape, one CUDA graph per
  chunk) against the plain per-trajectory loop (one funcutils.repeated call per
  trajectory, same GPU, same states).  Returns the JSON sub-object."""
  import torch  # pylint: disable=import-outside-toplevel
  import jax_cfd_gb300.base as cfd  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300 import batching, plans  # pylint: disable=import-outside-toplevel
  draws = ensemble_draws(args.ensemble_members)
  steps = args.ensemble_steps
  members, states = [], []
  for d in draws:
    grid = cfd.grids.Grid((d['n'], d['n']), domain=DOMAIN)
    members.append(batching.kolmogorov_member((d['n'], d['n']), d['nu'], d['dt'], d['k']))
    v0 = cfd.initial_conditions.filtered_velocity_field(d['seed'], grid, d['vmax'], 4,
                                                        device=dev)
    states.append((v0[0].data.clone(), v0[1].data.clone()))
  stream = torch.cuda.current_stream(dev)
  cells = sum(d['n'] ** 2 for d in draws)

  ens = batching.FvmEnsemble(members, device=dev)
  for i, (u, v) in enumerate(states):
    ens.set_state(i, u, v)
  ens.autotune(10)

  def load_all():
    for i, (u, v) in enumerate(states):
      ens.set_state(i, u, v)

  ens.step(steps, graph=True)  # capture + warm-up
  ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
  ens_ms = []
  for _ in range(2):
    load_all()
    flush.zero_()
    ev[0].record(stream)
    ens.step(steps, graph=True)
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    ens_ms.append(ev[0].elapsed_time(ev[1]))
  health = ens.health()  # per-member device health records after the last chunk
  finite_mask = [not (int(f) & 1) for f in health['flags']]

  # Plain loop: each trajectory through its own plan, one after another.
  plain_plans = []
  for m, (u, v) in zip(members, states):
    kw = dict(m)
    shape, step = kw.pop('shape'), kw.pop('step')
    pl = plans.FvmPlan(shape, step, device=dev, **kw)
    pl.autotune(u, v, 5)
    plain_plans.append(pl)
  outs = [(torch.empty_like(u), torch.empty_like(v)) for u, v in states]

  def plain():
    for pl, (u, v), (uo, vo) in zip(plain_plans, states, outs):
      pl.step(u, v, steps, uo, vo)

  plain()
  torch.cuda.synchronize(dev)
  plain_ms = []
  for _ in range(2):
    flush.zero_()
    ev[2].record(stream)
    plain()
    ev[3].record(stream)
    torch.cuda.synchronize(dev)
    plain_ms.append(ev[2].elapsed_time(ev[3]))
  def bits(t):
    return t.view(torch.int32)
  fin = [i for i in range(len(draws)) if finite_mask[i]]
  nonfin = [i for i in range(len(draws)) if not finite_mask[i]]
  # Finite members: bit for bit; non-finite ones: the plain loop is
  # non-finite too (NaN payloads are not compared).
  same = all(torch.equal(bits(ens.state(i)[0]), bits(outs[i][0])) and
             torch.equal(bits(ens.state(i)[1]), bits(outs[i][1])) for i in fin)
  plain_nonfinite_too = all(not (bool(torch.isfinite(outs[i][0]).all()) and
                                 bool(torch.isfinite(outs[i][1]).all())) for i in nonfin)
  flags_match_states = all(
      finite_mask[i] == (bool(torch.isfinite(ens.state(i)[0]).all()) and
                         bool(torch.isfinite(ens.state(i)[1]).all())) for i in range(len(draws)))
  fin_cells = sum(draws[i]['n'] ** 2 for i in fin)
  e_s, p_s = min(ens_ms) / 1000.0, min(plain_ms) / 1000.0
  sizes = {}
  for d in draws:
    sizes[d['n']] = sizes.get(d['n'], 0) + 1
  return {
      'workload': f'ragged FVM ensemble: {len(draws)} trajectories x {steps} steps, N in '
                  '{64..1024} uniform, nu log-uniform [1e-4, 1e-2], k in {2,4,8}, '
                  'vmax in [1, 4], own stable dt',
      'members_per_size': {str(k): v for k, v in sorted(sizes.items())},
      'value': len(draws) * steps / e_s, 'unit': 'trajectory-steps/s',
      'cell_steps_per_s': cells * steps / e_s,
      'ms': e_s * 1000.0,
      'plain_loop': {'value': len(draws) * steps / p_s, 'unit': 'trajectory-steps/s',
                     'cell_steps_per_s': cells * steps / p_s, 'ms': p_s * 1000.0,
                     'launches': len(draws) * (4 * steps + 1)},
      'speedup_vs_plain': p_s / e_s,
      'batches': ens.num_batches,
      'graph_launches_per_chunk': 1,
      # per batch: 4 per step, project_out, and the two health kernels
      'kernel_launches': ens.num_batches * (4 * steps + 3),
      'health': {'finite_members': len(fin), 'nonfinite_members': len(nonfin),
                 'flags_match_states': bool(flags_match_states),
                 'finite_trajectory_steps_per_s': len(fin) * steps / e_s,
                 'finite_cell_steps_per_s': fin_cells * steps / e_s,
                 'note': 'members whose explicit scheme leaves its stability region within '
                         'the horizon at their stable dt (both paths); flagged per member by '
                         'the device health records'},
      'bitwise_equal_to_plain_finite_members': bool(same),
      'plain_nonfinite_for_the_same_members': bool(plain_nonfinite_too),
  }


def run_serving(dev, args):
  """Continuous-batching server on a seeded Poisson stream (FVM and spectral
  requests, 100-step chunks, 150 GB budget); p50/p99 completion latency and
  throughput.  A short stream over every (kind, size) warms the per-size plans
  and the CUDA modules first; the timed server starts empty."""
  import torch  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300 import serving  # pylint: disable=import-outside-toplevel
  warm = []
  for i, (kind, n) in enumerate((kd, n) for kd in ('fvm', 'spectral') for n in serving.SIZES):
    for k in (2, 4, 8):
      warm.append(serving.Request(rid=10 ** 6 + 3 * i + k, kind=kind, n=n, steps=2,
                                  viscosity=1e-3, k=k, vmax=2.0, seed=1, arrival=0.0))
  serving.Server(device=dev, chunk=args.serve_chunk).serve(warm, realtime=False)
  reqs = serving.poisson_requests(args.serve_rate, args.serve_seconds, seed=7)
  server = serving.Server(device=dev, chunk=args.serve_chunk, budget_bytes=150e9)
  t0 = time.perf_counter()
  done = server.serve(reqs, realtime=True, timeout=args.serve_seconds + 600)
  makespan = time.perf_counter() - t0
  torch.cuda.synchronize(dev)
  st = serving.Server.stats(done, makespan)
  offered = sum(r.steps * r.n * r.n for r in reqs) / args.serve_seconds
  # Plain loop on the same request mix: one request after another through the
  # drop-in step (initial condition, funcutils.repeated, result to the host).
  plain_reqs = [serving.Request(rid=r.rid, kind=r.kind, n=r.n, steps=r.steps,
                                viscosity=r.viscosity, k=r.k, vmax=r.vmax, seed=r.seed)
                for r in reqs[:args.serve_plain]]
  t1 = time.perf_counter()
  for r in plain_reqs:
    serving.run_plain(r, dev)
  torch.cuda.synchronize(dev)
  plain_s = time.perf_counter() - t1
  plain_steps = sum(r.steps for r in plain_reqs)
  kinds = {}
  for kind in ('fvm', 'spectral'):
    sub = [r for r in done if r.kind == kind]
    lat = np.array([r.latency for r in sub])
    kinds[kind] = {'requests': len(sub),
                   'p50_latency_s': float(np.percentile(lat, 50)),
                   'p99_latency_s': float(np.percentile(lat, 99))}
  return {
      'workload': f'Poisson arrivals {args.serve_rate:g}/s for {args.serve_seconds:g} s; '
                  'FVM or spectral 50/50; N in {64..2048} with P(N) ~ 1/N^2; horizon '
                  'log-uniform 100-5000 steps; nu log-uniform [1e-4, 1e-2]; k in {2,4,8}; '
                  f'{args.serve_chunk}-step chunks; 150 GB budget',
      **st,
      'unit': 'trajectory-steps/s',
      'offered_cell_steps_per_s': offered,
      'plain_loop': {'requests': len(plain_reqs), 'seconds': plain_s,
                     'trajectory_steps_per_s': plain_steps / plain_s,
                     'sample': f'the first {len(plain_reqs)} requests of the stream, '
                               'one after another'},
      'speedup_vs_plain': st['trajectory_steps_per_s'] / (plain_steps / plain_s),
      'by_kind': kinds,
      'pools': sum(len(p) for p in server.pools.values()),
      'pool_bytes': server.bytes_in_use,
      'chunk_launches': server.launches,
  }


def run_differentiation(dev, args):
  """Gradient of a vorticity-matching loss through 64 FVM steps at 512^2 for
  a batch of 8 trajectories (seeds 0-7; targets from seeds 100-107 advanced
  64 steps), with respect to the initial velocities and the viscosity, by the
  hand-written adjoint with a checkpoint every 8 steps; timed forward +
  backward, and a finite-difference spot check along random directions with
  the float32 forward (eps 1e-3, 1e-4 and 1e-5)."""
  import torch  # pylint: disable=import-outside-toplevel
  import jax_cfd_gb300.base as cfd  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300 import adjoint  # pylint: disable=import-outside-toplevel
  n, batch, steps, every, nu0 = 512, 8, 64, 8, 1e-3
  grid = cfd.grids.Grid((n, n), domain=DOMAIN)
  dt = cfd.equations.stable_time_step(MAX_VELOCITY, CFL, nu0, grid)
  step = cfd.equations.semi_implicit_navier_stokes(
      1.0, nu0, dt, grid, forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1))
  spec = adjoint.spec_for(step, steps, checkpoint_every=every)

  def ic(seed):
    v = cfd.initial_conditions.filtered_velocity_field(seed, grid, MAX_VELOCITY, 4, device=dev)
    return v[0].data, v[1].data
  init = [ic(b) for b in range(batch)]
  u0 = torch.stack([a for a, _ in init]).contiguous()
  v0 = torch.stack([b for _, b in init]).contiguous()
  with torch.no_grad():
    tgt = [ic(100 + b) for b in range(batch)]
    tu, tv = adjoint.rollout(torch.stack([a for a, _ in tgt]), torch.stack([b for _, b in tgt]),
                             nu0, spec)
    target = adjoint.vorticity(tu, tv, grid.step)

  def loss_fn(u, v, nu):
    a, b = adjoint.rollout(u, v, nu, spec)
    return ((adjoint.vorticity(a, b, grid.step) - target) ** 2).mean()

  stream = torch.cuda.current_stream(dev)
  ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
  ms = []
  for rep in range(4):
    u = u0.clone().requires_grad_()
    v = v0.clone().requires_grad_()
    nu = torch.tensor(nu0, device=dev, requires_grad=True)
    ev[0].record(stream)
    loss = loss_fn(u, v, nu)
    loss.backward()
    ev[1].record(stream)
    torch.cuda.synchronize(dev)
    if rep:
      ms.append(ev[0].elapsed_time(ev[1]))
  gu, gv, gnu = u.grad, v.grad, float(nu.grad)
  rng = np.random.default_rng(0)
  eps = 1e-3

  def loss_difference(ua, va, nua, ub, vb, nub):
    """L(a) - L(b) from the two float32 rollouts, formed in float64 as
    mean((w_a - w_b) (w_a + w_b - 2 target)): the same quantity as the
    difference of the two losses, without the cancellation of subtracting
    two nearly equal float32 losses."""
    wa = adjoint.vorticity(*adjoint.rollout(ua, va, nua, spec), grid.step).double()
    wb = adjoint.vorticity(*adjoint.rollout(ub, vb, nub, spec), grid.step).double()
    return float(((wa - wb) * (wa + wb - 2 * target.double())).mean())

  eps_list = (eps, 1e-4, 1e-5)
  ads, fds = [], {e: [] for e in eps_list}
  with torch.no_grad():
    for _ in range(args.diff_directions):
      # Directions with unit RMS per cell, so that eps perturbs every cell by
      # about eps (a unit-norm direction over 2M cells would vanish below
      # float32 resolution).
      du = torch.from_numpy(rng.standard_normal(u0.shape).astype(np.float32)).to(dev)
      dv = torch.from_numpy(rng.standard_normal(v0.shape).astype(np.float32)).to(dev)
      ads.append(float((gu.double() * du.double()).sum() + (gv.double() * dv.double()).sum()))
      for e in eps_list:
        fds[e].append(loss_difference(u0 + e * du, v0 + e * dv, nu0,
                                      u0 - e * du, v0 - e * dv, nu0) / (2 * e))
    hn = 1e-6
    fd_nu = loss_difference(u0, v0, nu0 + hn, u0, v0, nu0 - hn) / (2 * hn)
  ad_arr = np.asarray(ads)
  ad_rms = float(np.sqrt(np.mean(ad_arr ** 2))) if ads else 0.0

  def fd_stats(e):
    err = np.abs(np.asarray(fds[e]) - ad_arr)
    rel = err / np.maximum(np.abs(ad_arr), 1e-30)
    return {'max_rel_err': float(rel.max()), 'median_rel_err': float(np.median(rel)),
            'max_err_over_rms': float(err.max() / max(ad_rms, 1e-30))}

  errs = fd_stats(eps) if ads else {}
  t = float(np.median(ms)) / 1000.0
  return {
      'workload': f'loss = MSE(vorticity after {steps} FVM steps, target) at {n}x{n}, batch '
                  f'{batch}; gradient wrt initial velocity and viscosity; checkpoint every {every}',
      'forward_backward_ms': t * 1000.0,
      'trajectory_steps_per_s': batch * steps / t,
      'cell_steps_per_s': batch * steps * n * n / t,
      'loss': float(loss.detach()),
      'fd_check': {'directions': len(ads), 'eps': eps, 'direction_rms': 1.0,
                   'max_rel_err': errs.get('max_rel_err'),
                   'median_rel_err': errs.get('median_rel_err'),
                   'max_err_over_rms': errs.get('max_err_over_rms'),
                   'viscosity_rel_err': abs(gnu - fd_nu) / max(abs(fd_nu), 1e-30),
                   'forward': 'float32 GPU rollouts, loss difference formed in float64',
                   'by_eps': {f'{e:g}': fd_stats(e) for e in eps_list} if ads else {},
                   'note': 'rel_err = |fd - ad| / |ad| per direction, so its maximum is set '
                           'by the direction with the smallest |ad|; max_err_over_rms '
                           'divides by the RMS of ad over the directions.  eps perturbs '
                           'every cell by about eps and crosses Van Leer limiter kinks '
                           '(r = 0), where the derivative jumps'},
      'batch_execution': 'the 8 trajectories run concurrently, one plan and stream each',
      'targets': 'vorticity of this path advanced 64 steps from seeds 100-107 (the oracle '
                 'runs only in tests; tests/test_gpu_adjoint.py takes its target from the '
                 'float64 restatement)',
  }


def run_gb300(args):
  import torch  # pylint: disable=import-outside-toplevel
  import jax_cfd_gb300.base as cfd  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300 import plans  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.spectral import equations as seq  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.spectral import time_stepping as sts  # pylint: disable=import-outside-toplevel

  world, rank, local = _dist()
  torch.cuda.set_device(local)
  dev = torch.device('cuda', local)
  dist = None
  if world > 1:
    import torch.distributed as dist  # pylint: disable=import-outside-toplevel
    dist.init_process_group('nccl', device_id=dev)

  def barrier():
    if dist is not None:
      dist.barrier()

  n, chunk = args.size, args.chunk
  grid = cfd.grids.Grid((n, n), domain=DOMAIN)
  v0 = cfd.initial_conditions.filtered_velocity_field(rank, grid, MAX_VELOCITY, 4, device=dev)
  dt = cfd.equations.stable_time_step(MAX_VELOCITY, CFL, VISCOSITY, grid)
  forcing = cfd.forcings.simple_turbulence_forcing(grid, 1, 4, -0.1)
  step = cfd.equations.semi_implicit_navier_stokes(1.0, VISCOSITY, dt, grid, forcing=forcing)
  run = cfd.funcutils.repeated(step, chunk)
  flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
  stream = torch.cuda.current_stream(dev)

  # Every bench step advances the same seeded initial condition by `chunk`
  # steps.  (A single 2000-step trajectory of this configuration leaves the
  # explicit scheme's stability region: the forcing accelerates the flow past
  # the speed dt was chosen for, and the reference algorithm overflows near
  # t = 0.9 at 2048^2 -- the oracle and this path blow up at the same step.)
  plan = step.plan(dev)
  if args.launch >= 0:
    plan.set_launch(args.launch)
    shape = args.launch
  else:
    shape = plan.autotune(v0[0].data, v0[1].data, 20)
  v = v0
  for _ in range(args.warmup):
    v = run(v0)
  torch.cuda.synchronize(dev)

  starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  sampler = ClockSampler(local)
  barrier()
  torch.cuda.synchronize(dev)
  with sampler:
    t0 = time.perf_counter()
    for k in range(args.steps):
      flush.zero_()
      starts[k].record(stream)
      v = run(v0)
      ends[k].record(stream)
    torch.cuda.synchronize(dev)
    wall = time.perf_counter() - t0
  barrier()
  chunk_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
  total_s = max_over_ranks(sum(chunk_ms) / 1000.0)
  cells = n * n
  value = world * cells * chunk * args.steps / total_s
  finite = bool(torch.isfinite(v[0].data).all() and torch.isfinite(v[1].data).all())

  # Per-kernel durations (second pass, same workload and state).
  kernel_ms = plan.profile(v0[0].data, v0[1].data, chunk)
  kernel_time = {k: kernel_ms[k] * (chunk if k != 'project_out' else 1) for k in kernel_ms}
  dominant = max(kernel_time, key=kernel_time.get)
  peak, peak_kind = _peaks()
  achieved = FVM_BYTES_PER_CELL[dominant] * cells / (kernel_ms[dominant] / 1000.0) / 1e9
  traffic = _traffic_table().get(f'fvm_{dominant}_{n}')
  step_achieved = FVM_STEP_BYTES_PER_CELL * value / world / 1e9

  # End to end through the public API with host buffers.
  host_u = torch.empty((n, n), dtype=torch.float32, pin_memory=True)
  host_v = torch.empty((n, n), dtype=torch.float32, pin_memory=True)
  host_u.copy_(v0[0].data)
  host_v.copy_(v0[1].data)
  out_u = torch.empty_like(host_u, pin_memory=True)
  out_v = torch.empty_like(host_v, pin_memory=True)
  bc = cfd.boundaries.periodic_boundary_conditions(2)
  e2e_steps = max(1, min(args.steps, 5))
  e_start = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps)]
  e_end = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps)]
  torch.cuda.synchronize(dev)
  for k in range(e2e_steps):
    flush.zero_()
    e_start[k].record(stream)
    du = host_u.to(dev, non_blocking=True)
    dv = host_v.to(dev, non_blocking=True)
    state = (cfd.grids.GridVariable(cfd.grids.GridArray(du, grid.cell_faces[0], grid), bc),
             cfd.grids.GridVariable(cfd.grids.GridArray(dv, grid.cell_faces[1], grid), bc))
    res = run(state)
    out_u.copy_(res[0].data, non_blocking=True)
    out_v.copy_(res[1].data, non_blocking=True)
    e_end[k].record(stream)
  torch.cuda.synchronize(dev)
  e2e_s = sum(s.elapsed_time(e) for s, e in zip(e_start, e_end)) / 1000.0
  e2e_value = world * cells * chunk * e2e_steps / e2e_s

  # The same through the public API with the host copies around every single
  # time step (the drop-in step called once per time step), for comparison.
  one = 20
  o_start = torch.cuda.Event(enable_timing=True)
  o_end = torch.cuda.Event(enable_timing=True)
  torch.cuda.synchronize(dev)
  o_start.record(stream)
  for _ in range(one):
    du = host_u.to(dev, non_blocking=True)
    dv = host_v.to(dev, non_blocking=True)
    state = (cfd.grids.GridVariable(cfd.grids.GridArray(du, grid.cell_faces[0], grid), bc),
             cfd.grids.GridVariable(cfd.grids.GridArray(dv, grid.cell_faces[1], grid), bc))
    res = step(state)
    out_u.copy_(res[0].data, non_blocking=True)
    out_v.copy_(res[1].data, non_blocking=True)
  o_end.record(stream)
  torch.cuda.synchronize(dev)
  e2e_one_value = world * cells * one / (o_start.elapsed_time(o_end) / 1000.0)

  # Secondary: the pseudospectral step at the same size (CN-RK4, dt = 1e-3).
  spectral = None
  if not args.skip_spectral:
    from jax_cfd_gb300.spectral import utils as su  # pylint: disable=import-outside-toplevel
    w0 = su.rfft2(cfd.finite_differences.curl_2d(v0).data, grid)
    eq = seq.ForcedNavierStokes2D(VISCOSITY, grid, smooth=True)
    sstep = sts.crank_nicolson_rk4(eq, 1e-3)
    splan = sstep.plan(dev)
    s_launch = splan.autotune(w0, 4) if args.spectral_launch < 0 else args.spectral_launch
    splan.set_launch(s_launch)
    srun = cfd.funcutils.repeated(sstep, args.spectral_chunk)
    for _ in range(3):
      w = srun(w0)
    torch.cuda.synchronize(dev)
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s_ms = 0.0
    for _ in range(3):
      flush.zero_()
      s0.record(stream)
      w = srun(w0)
      s1.record(stream)
      torch.cuda.synchronize(dev)
      s_ms += s0.elapsed_time(s1)
    s_value = cells * args.spectral_chunk * 3 / (s_ms / 1000.0)
    sk = sstep.plan(dev).profile(w0, 2)
    s_per_step = spectral_launches_per_time_step(args.spectral_chunk)
    s_dom = spectral_dominant_kernel(sk, args.spectral_chunk)
    s_ach = SPEC_BYTES_PER_CELL[s_dom] * cells / (sk[s_dom] / 1000.0) / 1e9
    spectral = {
        'workload': f'NavierStokes2D {n}x{n} crank_nicolson_rk4 dt=1e-3, Kolmogorov k=4, drag 0.1',
        'value': s_value, 'unit': 'cell-steps/s',
        'ms_per_time_step': s_ms / (3 * args.spectral_chunk),
        'step_roofline': {'bytes_per_cell_step': SPEC_STEP_BYTES_PER_CELL,
                          'achieved': SPEC_STEP_BYTES_PER_CELL * s_value / 1e9,
                          'peak': peak, 'unit': 'GB/s',
                          'frac': SPEC_STEP_BYTES_PER_CELL * s_value / 1e9 / peak},
        'kernel_ms': sk,
        'column_pass': splan.COLUMN_PASSES[s_launch % 5],
        'row_pass': splan.ROW_PASSES[s_launch // 5],
        'launches_per_time_step': s_per_step,
        'roofline': {'kernel': s_dom, 'bound': 'hbm', 'achieved': s_ach, 'peak': peak,
                     'unit': 'GB/s', 'frac': s_ach / peak,
                     'traffic': _traffic_table().get(f'spec_{s_dom}_{n}')},
        'finite': bool(torch.isfinite(torch.view_as_real(w)).all()),
    }

  ensemble = None
  if not args.skip_ensemble:
    ensemble = run_ensemble(dev, args, flush)

  differentiation = None
  if not args.skip_diff:
    differentiation = run_differentiation(dev, args)

  served = None
  if not args.skip_serving:
    served = run_serving(dev, args)

  cpu = None
  if rank == 0 and not args.skip_cpu:
    cv, csecs, cthreads = _cpu_sample(args.cpu_steps, 1)
    cpu = {'value': cv, 'unit': 'cell-steps/s', 'cores': cthreads, 'kind': 'port',
           'sample': f'{cthreads} host processes (one per core), each {args.cpu_steps} FVM '
                     f'steps of its own {N}x{N} trajectory of the NumPy restatement after 1 '
                     f'warm-up step ({csecs:.1f} s)'}

  if rank != 0:
    return
  launches = args.steps * (4 * chunk + 1)
  _json_line({
      'metric': 'FVM cell-steps/s at 2048^2', 'value': value, 'unit': 'cell-steps/s',
      'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
      'ms_per_step': 1000.0 * total_s / args.steps, 'higher_is_better': True,
      'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
      'config': {'workload': fvm_workload(n), 'grid': [n, n], 'time_steps_per_step': chunk,
                 'dt': dt,
                 'l2': 'flushed (256 MiB write) between bench steps',
                 'launch_config': plans.FvmPlan.describe_launch(shape),
                 'parallelism': 'replicas' if world > 1 else 'single'},
      'roofline': {'kernel': dominant, 'bound': 'hbm', 'achieved': achieved, 'peak': peak,
                   'unit': 'GB/s', 'frac': achieved / peak, 'traffic': traffic,
                   'peak_source': peak_kind,
                   'bytes_per_cell': FVM_BYTES_PER_CELL[dominant]},
      'step_roofline': {'bytes_per_cell_step': FVM_STEP_BYTES_PER_CELL,
                        'achieved': step_achieved, 'peak': peak, 'unit': 'GB/s',
                        'frac': step_achieved / peak},
      'kernel_ms': kernel_ms,
      'cpu_baseline': cpu,
      'e2e': {'value': e2e_value, 'unit': 'cell-steps/s',
              'h2d_bytes_per_step': 2 * cells * 4, 'd2h_bytes_per_step': 2 * cells * 4},
      'e2e_per_time_step': {'value': e2e_one_value, 'unit': 'cell-steps/s',
                            'h2d_bytes_per_time_step': 2 * cells * 4,
                            'd2h_bytes_per_time_step': 2 * cells * 4,
                            'note': 'the drop-in step called once per time step with the '
                                    'pinned host state copied in and out around every call'},
      'gpu_launches': launches,
      'clocks': sampler.summary(),
      'wall_s': wall,
      'finite': finite,
      'spectral': spectral,
      'ensemble': ensemble,
      'serving': served,
      'differentiation': differentiation,
  })


def main():
  ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
  ap.add_argument('--gpus', type=int, default=1)
  ap.add_argument('--steps', type=int, default=10)
  ap.add_argument('--warmup', type=int, default=3)
  ap.add_argument('--impl', choices=['gb300', 'reference'], default='gb300')
  ap.add_argument('--size', type=int, default=N)
  ap.add_argument('--chunk', type=int, default=200)
  ap.add_argument('--launch', type=int, default=-1,
                  help='pin the FVM launch configuration (default: autotune)')
  ap.add_argument('--spectral-chunk', type=int, default=20)
  ap.add_argument('--spectral-launch', type=int, default=-1,
                  help='pin the spectral column-pass scheme (default: autotune)')
  ap.add_argument('--cpu-steps', type=int, default=5)
  ap.add_argument('--skip-cpu', action='store_true')
  ap.add_argument('--skip-spectral', action='store_true')
  ap.add_argument('--skip-ensemble', action='store_true')
  ap.add_argument('--ensemble-members', type=int, default=96)
  ap.add_argument('--ensemble-steps', type=int, default=1000)
  ap.add_argument('--skip-serving', action='store_true')
  ap.add_argument('--serve-rate', type=float, default=200.0)
  ap.add_argument('--serve-seconds', type=float, default=60.0)
  ap.add_argument('--serve-chunk', type=int, default=100)
  ap.add_argument('--serve-plain', type=int, default=150)
  ap.add_argument('--skip-diff', action='store_true')
  ap.add_argument('--diff-directions', type=int, default=32)
  args = ap.parse_args()
  if args.warmup < 3:
    ap.error('at least 3 warm-up steps are required')
  if args.impl == 'reference':
    run_reference(args)
  else:
    run_gb300(args)


if __name__ == '__main__':
  main()
