"""Continuous-batching simulation server over the batched FVM and spectral
steps.

Requests (grid size, viscosity, forcing wavenumber, horizon, seed; FVM
``semi_implicit_navier_stokes`` or spectral ``NavierStokes2D`` +
``crank_nicolson_rk4``) arrive over time.  Each request's state lives in a slot
of a device-resident *pool* -- a same-shape batch (``batching.FvmBatch`` or
``batching.SpecBatch``) with its own CUDA stream -- from admission to
completion.  Pools advance in chunks of ``chunk`` steps, one CUDA-graph launch
per chunk; every pool cycles independently:

    chunk done -> retire finished slots (result copied to pinned host memory)
               -> admit queued requests into free slots (initial condition
                  generated on the device, slot parameters set)
               -> launch the next chunk with each slot's remaining steps

so requests that arrive while others are on the GPU join at the next chunk
boundary of a pool of their size, and work of different pools overlaps on the
device.  New pools are allocated on demand while the total pool memory stays
within ``budget_bytes``; otherwise requests wait in their size's queue.

Reported per request: arrival, admission and completion times (completion =
result on the host); ``Server.stats`` gives p50/p99 latency and throughput.
A request's result does not depend on which other requests share its pool.

Health: every chunk ends with a per-slot reduction on the device (non-finite
flag and largest finite magnitude of the state, ``cfd_health``), which the
chunk's last kernel also writes into the pool's pinned host buffer.  A request whose state holds a NaN or an infinity, or
whose FVM velocity exceeds ``max_speed_factor`` times its initial maximum
speed, is retired at that chunk boundary with ``status`` 'nonfinite' or
'diverged', an ``error`` message and no result array, and its slot is freed.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

HEALTH_NONFINITE = 1  # cfd_health flag: the state holds NaN or infinity
TWO_PI = 2 * math.pi
CFL = 0.5
DRAG = 0.1
SIZES = (64, 128, 256, 512, 1024, 2048)


@dataclasses.dataclass
class Request:
  """One simulation request.  ``dt`` follows the kind: FVM takes
  stable_time_step(vmax, 0.5, nu) or, where the reference would raise, the
  diffusive limit h^2 / (4 nu); the spectral step treats diffusion implicitly
  and takes the advective limit 0.5 h / vmax."""
  rid: int
  kind: str          # 'fvm' or 'spectral'
  n: int             # grid is n x n on [0, 2 pi]^2
  steps: int
  viscosity: float
  k: int             # Kolmogorov forcing wavenumber
  vmax: float        # max speed of the initial velocity
  seed: int
  arrival: float = 0.0     # seconds after the stream starts
  admitted: Optional[float] = None
  finished: Optional[float] = None
  result: Optional[Tuple[np.ndarray, ...]] = None
  status: str = 'pending'  # 'ok', 'nonfinite' or 'diverged' once finished
  error: Optional[str] = None
  dt_override: Optional[float] = None  # replaces the stable dt when given

  @property
  def dt(self) -> float:
    if self.dt_override is not None:
      return float(self.dt_override)
    h = TWO_PI / self.n
    if self.kind == 'fvm':
      return min(CFL * h / self.vmax, h * h / (4 * self.viscosity))
    return CFL * h / self.vmax

  @property
  def latency(self) -> Optional[float]:
    return None if self.finished is None else self.finished - self.arrival


def size_weights(sizes: Sequence[int] = SIZES) -> np.ndarray:
  """P(N) proportional to 1/N^2: small grids are the most frequent and every
  size carries the same expected number of cells."""
  w = np.array([1.0 / (n * n) for n in sizes])
  return w / w.sum()


def poisson_requests(rate: float, duration: float, seed: int = 0,
                     sizes: Sequence[int] = SIZES, min_steps: int = 100,
                     max_steps: int = 5000) -> List[Request]:
  """A seeded Poisson arrival stream: FVM or spectral with probability 1/2,
  N from `sizes` with size_weights, horizon log-uniform in [min_steps,
  max_steps], viscosity log-uniform in [1e-4, 1e-2], k in {2, 4, 8}, vmax
  uniform in [1, 4], seed = request id."""
  rng = np.random.default_rng(seed)
  p = size_weights(sizes)
  out, t, rid = [], 0.0, 0
  while True:
    t += rng.exponential(1.0 / rate)
    if t >= duration:
      break
    out.append(Request(
        rid=rid, kind='fvm' if rng.random() < 0.5 else 'spectral',
        n=int(rng.choice(sizes, p=p)),
        steps=int(round(math.exp(rng.uniform(math.log(min_steps), math.log(max_steps))))),
        viscosity=float(10 ** rng.uniform(-4, -2)), k=int(rng.choice([2, 4, 8])),
        vmax=float(rng.uniform(1, 4)), seed=rid, arrival=t))
    rid += 1
  return out


def default_capacity(kind: str, n: int) -> int:
  """Slots per pool: about 2^21 cells per pool, between 2 and 16 slots."""
  del kind
  return int(min(16, max(2, (1 << 21) // (n * n))))


# Spectral forcing curl tables per (device, N, k), shared by every server.
_FORCING_PLANS = {}


class _Pool:
  """One same-shape batch, its stream and slot bookkeeping."""

  def __init__(self, server: 'Server', kind: str, n: int, capacity: int):
    from jax_cfd_gb300 import batching  # pylint: disable=import-outside-toplevel
    from jax_cfd_gb300.base import grids  # pylint: disable=import-outside-toplevel
    self.kind, self.n, self.capacity = kind, n, capacity
    self.grid = grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
    dev = server.device
    if kind == 'fvm':
      self.batch = batching.FvmBatch((n, n), self.grid.step, capacity, device=dev)
    else:
      self.batch = batching.SpecBatch((n, n), self.grid.step, capacity, device=dev)
    self.stream = torch.cuda.Stream(dev)
    # Health records of the last chunk, written into pinned memory by the
    # chunk's last kernel (no device-to-host copy behind other transfers).
    self.health_host = torch.zeros((capacity, 2), dtype=torch.int32, pin_memory=True)
    self.batch.set_health_mirror(self.health_host)
    self.slots: List[Optional[Request]] = [None] * capacity
    self.remaining = [0] * capacity
    self.running = [0] * capacity
    self.event: Optional[torch.cuda.Event] = None
    self.nbytes = self.batch.nbytes

  def active(self) -> bool:
    return any(r is not None for r in self.slots)

  def release(self):
    """Returns the pool's device memory (synchronises the device)."""
    torch.cuda.synchronize(self.batch.device)
    self.batch = None


class Server:
  """The request loop (single host thread, one GPU)."""

  def __init__(self, device=None, budget_bytes: float = 150e9, chunk: int = 100,
               graph: bool = True, capacity=default_capacity,
               max_speed_factor: float = 100.0, check_health: bool = True):
    self.device = torch.device(device) if device is not None else torch.device(
        'cuda', torch.cuda.current_device())
    self.budget = float(budget_bytes)
    self.chunk = int(chunk)
    self.graph = graph
    self.capacity = capacity
    self.max_speed_factor = float(max_speed_factor)
    self.check_health = bool(check_health)
    self.pools: Dict[Tuple[str, int], List[_Pool]] = collections.defaultdict(list)
    self.queues: Dict[Tuple[str, int], collections.deque] = collections.defaultdict(
        collections.deque)
    self.bytes_in_use = 0
    self.admit_stream = torch.cuda.Stream(self.device)
    self._retiring: List[tuple] = []  # (request, copy event, host arrays, pool)
    self._forcing_plans = _FORCING_PLANS
    self.done: List[Request] = []
    self.t0 = None
    self.launches = 0

  # -- clock ---------------------------------------------------------------
  def now(self) -> float:
    return time.perf_counter() - self.t0

  # -- admission -----------------------------------------------------------
  def submit(self, req: Request):
    self.queues[(req.kind, req.n)].append(req)

  def _pool_with_room(self, key):
    """(pool, slot) of a free slot in a pool between chunks; 'wait' when the
    only free slots are in pools whose chunk is still running (they open at
    its end); None when every pool of this size is full."""
    wait = False
    for pool in self.pools[key]:
      for i, r in enumerate(pool.slots):
        if r is None:
          if pool.event is None:
            return pool, i
          wait = True
          break
    return 'wait' if wait else None

  def _evict_idle(self, need: int, keep) -> bool:
    """Frees empty pools of other sizes (between chunks, no result copy
    pending) until `need` more bytes fit in the budget."""
    pending = {id(p) for p in self._copying}
    for key, pools in self.pools.items():
      if key == keep:
        continue
      for pool in list(pools):
        if self.bytes_in_use + need <= self.budget:
          return True
        if pool.event is None and not pool.active() and id(pool) not in pending:
          pools.remove(pool)
          self.bytes_in_use -= pool.nbytes
          pool.release()
    return self.bytes_in_use + need <= self.budget

  def _new_pool(self, key) -> Optional[_Pool]:
    kind, n = key
    cap = self.capacity(kind, n)
    need = cap * self.slot_bytes(kind, n)
    if self.bytes_in_use + need > self.budget and not self._evict_idle(need, key):
      if not any(p.active() or p.event is not None for ps in self.pools.values() for p in ps):
        raise MemoryError(f'a {kind} pool of {cap} slots at {n}^2 needs {need} bytes; '
                          f'the budget is {self.budget:.0f}')
      return None
    pool = _Pool(self, kind, n, cap)
    self.bytes_in_use += pool.nbytes
    self.pools[key].append(pool)
    return pool

  @staticmethod
  def slot_bytes(kind: str, n: int) -> int:
    """Device bytes of one slot: FVM state, two step buffers and the pressure
    spectrum (7 n^2 floats) plus its forcing tables; spectral state, carry,
    four column fields and the advection spectra (7 half spectra)."""
    return (7 * n * n * 4 + 8 * n) if kind == 'fvm' else 7 * n * (n // 2 + 1) * 8

  def _spec_forcing_plan(self, n: int, k: int):
    key = (self.device, n, k)
    if key not in self._forcing_plans:
      from jax_cfd_gb300.base import forcings, grids  # pylint: disable=import-outside-toplevel
      from jax_cfd_gb300.spectral import equations as seq  # pylint: disable=import-outside-toplevel
      grid = grids.Grid((n, n), domain=((0, TWO_PI), (0, TWO_PI)))
      eq = seq.NavierStokes2D(0.0, grid, drag=DRAG, smooth=True,
                              forcing_fn=lambda g: forcings.kolmogorov_forcing(
                                  g, k=k, offsets=((0, 0), (0, 0))))
      self._forcing_plans[key] = eq._plan(self.device)  # pylint: disable=protected-access
    return self._forcing_plans[key]

  def _initial_state(self, req: Request, grid):
    """Device initial condition of a request (on the current stream)."""
    import jax_cfd_gb300.base as cfd  # pylint: disable=import-outside-toplevel
    v0 = cfd.initial_conditions.filtered_velocity_field(req.seed, grid, req.vmax, 4,
                                                        device=self.device)
    if req.kind == 'fvm':
      return v0[0].data, v0[1].data
    from jax_cfd_gb300.spectral import utils as su  # pylint: disable=import-outside-toplevel
    return (su.rfft2(cfd.finite_differences.curl_2d(v0).data, grid),)

  def _admit(self, pool: _Pool, slot: int, req: Request):
    from jax_cfd_gb300 import batching  # pylint: disable=import-outside-toplevel
    from jax_cfd_gb300.spectral import time_stepping as sts  # pylint: disable=import-outside-toplevel
    with torch.cuda.stream(self.admit_stream):
      state = self._initial_state(req, pool.grid)
      if req.kind == 'fvm':
        m = batching.kolmogorov_member((req.n, req.n), req.viscosity, req.dt, req.k)
        kw = dict(m)
        kw.pop('shape'), kw.pop('step')
        pool.batch.set_slot(slot, **kw)
        pool.batch.set_state(slot, *state)
      else:
        a, b, g = sts.CN_RK4_COEFFICIENTS
        pool.batch.set_slot(slot, viscosity=req.viscosity, drag=DRAG, dt=req.dt, smooth=True,
                            alphas=a, betas=b, gammas=g,
                            forcing_plan=self._spec_forcing_plan(req.n, req.k))
        pool.batch.set_state(slot, state[0])
    pool.slots[slot] = req
    pool.remaining[slot] = req.steps
    req.admitted = self.now()

  # -- the loop --------------------------------------------------------------
  def _unhealthy(self, req: Request, record) -> Optional[Tuple[str, str]]:
    """(status, message) when a slot's health record shows a failed state."""
    if record['flags'] & HEALTH_NONFINITE:
      return 'nonfinite', 'the state holds NaN or infinity'
    limit = self.max_speed_factor * req.vmax
    if req.kind == 'fvm' and record['max_abs'] > limit:
      return 'diverged', (f'velocity {float(record["max_abs"]):.3g} exceeds '
                          f'{self.max_speed_factor:g} x the initial maximum speed')
    return None

  def _finish_chunk(self, pool: _Pool):
    from jax_cfd_gb300 import batching  # pylint: disable=import-outside-toplevel
    health = batching.decode_health(pool.health_host)
    for i, req in enumerate(pool.slots):
      if req is None:
        continue
      ran = pool.running[i] > 0
      pool.remaining[i] -= pool.running[i]
      pool.running[i] = 0
      failed = self._unhealthy(req, health[i]) if ran and self.check_health else None
      if failed is not None:
        # Retire now with an error status: no result, the slot is freed.
        req.status, req.error = failed
        req.finished = self.now()
        self.done.append(req)
        pool.slots[i] = None
        continue
      if pool.remaining[i] <= 0:
        # Retire: copy the result to pinned host memory on the pool's stream.
        with torch.cuda.stream(pool.stream):
          dev = pool.batch.state(i)
          dev = dev if isinstance(dev, tuple) else (dev,)
          host = tuple(torch.empty(d.shape, dtype=d.dtype, pin_memory=True) for d in dev)
          for h, d in zip(host, dev):
            h.copy_(d, non_blocking=True)
          ev = torch.cuda.Event()
          ev.record(pool.stream)
        self._retiring.append((req, ev, host, pool))
        pool.slots[i] = None
    pool.event = None

  def _launch(self, pool: _Pool):
    for i, req in enumerate(pool.slots):
      steps = 0 if req is None else min(self.chunk, pool.remaining[i])
      pool.batch.set_steps(i, steps)
      pool.running[i] = steps
    # The chunk reads what admission wrote on the admission stream.
    ev = torch.cuda.Event()
    ev.record(self.admit_stream)
    pool.stream.wait_event(ev)
    with torch.cuda.stream(pool.stream):
      pool.batch.run(self.chunk, graph=self.graph)
      pool.event = torch.cuda.Event()
      pool.event.record(pool.stream)
    self.launches += 1

  def poll(self) -> bool:
    """One pass over the pools; returns whether anything happened."""
    progressed = False
    # Retire results whose copies completed.
    still = []
    for req, ev, host, pool in self._retiring:
      if ev.query():
        req.finished = self.now()
        req.result = tuple(h.numpy() for h in host)
        req.status = 'ok'
        self.done.append(req)
        progressed = True
      else:
        still.append((req, ev, host, pool))
    self._retiring = still
    # Chunks that finished.
    for pools in self.pools.values():
      for pool in pools:
        if pool.event is not None and pool.event.query():
          # Admission into this pool must not overwrite a slot whose result
          # copy is still queued on the pool's stream.
          self._finish_chunk(pool)
          ev = torch.cuda.Event()
          ev.record(pool.stream)
          self.admit_stream.wait_event(ev)
          progressed = True
    # Admission: fill idle pools' free slots, then open pools while memory allows.
    for key, queue in self.queues.items():
      while queue:
        room = self._pool_with_room(key)
        if room == 'wait':
          break
        if room is None:
          pool = self._new_pool(key)
          if pool is None:
            break
          room = (pool, 0)
        self._admit(room[0], room[1], queue.popleft())
        progressed = True
    # Launch idle pools that hold work.
    for pools in self.pools.values():
      for pool in pools:
        if pool.event is None and pool.active():
          self._launch(pool)
          progressed = True
    return progressed

  @property
  def _copying(self):
    return [entry[3] for entry in self._retiring]

  def busy(self) -> bool:
    return bool(self._retiring) or any(q for q in self.queues.values()) or any(
        p.active() or p.event is not None for ps in self.pools.values() for p in ps)

  def serve(self, requests: Sequence[Request], realtime: bool = True,
            timeout: float = 600.0) -> List[Request]:
    """Feeds `requests` at their arrival times (or all at once when
    realtime=False) and runs until every request finished."""
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    self.t0 = time.perf_counter()
    while pending or self.busy():
      now = self.now()
      if now > timeout:
        raise TimeoutError(f'serving did not finish within {timeout} s')
      while pending and (not realtime or pending[0].arrival <= now):
        self.submit(pending.popleft())
      if not self.poll():
        time.sleep(0.0002)
    return self.done

  # -- report ----------------------------------------------------------------
  @staticmethod
  def stats(done: Sequence[Request], makespan: float) -> dict:
    lat = np.array([r.latency for r in done])
    ok = [r for r in done if r.status == 'ok']
    steps = sum(r.steps for r in ok)
    cells = sum(r.steps * r.n * r.n for r in ok)
    return {
        'requests': len(done),
        'completed_ok': len(ok),
        'nonfinite': sum(r.status == 'nonfinite' for r in done),
        'diverged': sum(r.status == 'diverged' for r in done),
        'p50_latency_s': float(np.percentile(lat, 50)) if len(lat) else None,
        'p99_latency_s': float(np.percentile(lat, 99)) if len(lat) else None,
        'mean_latency_s': float(lat.mean()) if len(lat) else None,
        'makespan_s': makespan,
        'trajectory_steps_per_s': steps / makespan,
        'cell_steps_per_s': cells / makespan,
    }


def run_plain(req: Request, device=None) -> Request:
  """The plain path for one request: its initial condition, then
  ``funcutils.repeated`` of the drop-in step, then the result to the host."""
  import jax_cfd_gb300.base as cfd  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.base import forcings  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.spectral import equations as seq  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.spectral import time_stepping as sts  # pylint: disable=import-outside-toplevel
  from jax_cfd_gb300.spectral import utils as su  # pylint: disable=import-outside-toplevel
  dev = torch.device(device) if device is not None else torch.device(
      'cuda', torch.cuda.current_device())
  grid = cfd.grids.Grid((req.n, req.n), domain=((0, TWO_PI), (0, TWO_PI)))
  v0 = cfd.initial_conditions.filtered_velocity_field(req.seed, grid, req.vmax, 4, device=dev)
  if req.kind == 'fvm':
    step = cfd.equations.semi_implicit_navier_stokes(
        1.0, req.viscosity, req.dt, grid,
        forcing=cfd.forcings.simple_turbulence_forcing(grid, 1, req.k, -0.1))
    out = cfd.funcutils.repeated(step, req.steps)(v0)
    req.result = tuple(o.data.cpu().numpy() for o in out)
    req.status = 'ok'
  else:
    eq = seq.NavierStokes2D(req.viscosity, grid, drag=DRAG, smooth=True,
                            forcing_fn=lambda g: forcings.kolmogorov_forcing(
                                g, k=req.k, offsets=((0, 0), (0, 0))))
    w0 = su.rfft2(cfd.finite_differences.curl_2d(v0).data, grid)
    out = cfd.funcutils.repeated(sts.crank_nicolson_rk4(eq, req.dt), req.steps)(w0)
    req.result = (out.cpu().numpy(),)
    req.status = 'ok'
  return req

