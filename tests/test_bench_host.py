"""Host-side pieces of bench.py: which kernel the spectral roofline reports, and
that the DRAM-traffic table covers the kernels the roofline lines name."""
import importlib.util
import json
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
  spec = importlib.util.spec_from_file_location('bench_module', ROOT / 'bench.py')
  mod = importlib.util.module_from_spec(spec)
  spec.loader.exec_module(mod)
  return mod


def test_spectral_launches_per_time_step():
  b = _bench()
  per = b.spectral_launches_per_time_step(20)
  assert per['row'] == 5.0
  assert per['col_stage'] + per['col_update'] == 5.0
  assert per['col_prep'] == 1.0 / 20


def test_spectral_dominant_kernel_weighs_launches_per_step():
  b = _bench()
  # Per launch the prep is the longest, but it runs once per chunk.
  ms = {'row': 0.0423, 'col_stage': 0.0532, 'col_update': 0.0327, 'col_prep': 0.0639}
  assert b.spectral_dominant_kernel(ms, 20) == 'col_stage'
  assert b.spectral_dominant_kernel(dict(ms, row=0.060), 20) == 'row'
  # A one-step chunk: four fused stages, one update, one prep per step.
  assert b.spectral_dominant_kernel(dict(ms, col_prep=0.5), 1) == 'col_prep'


def test_traffic_table_covers_the_reported_kernels():
  b = _bench()
  table = b._traffic_table()  # pylint: disable=protected-access
  raw = json.loads((ROOT / 'profiles' / 'dram_traffic.json').read_text())
  assert table == raw
  for key in ('fvm_explicit_2048', 'spec_col_stage_2048', 'spec_row_2048'):
    assert isinstance(table[key], float) and table[key] > 0, key
  # DRAM bytes of one cold-cache launch stay below the algorithmic bytes
  # (20, 36 and 20 B per cell of a 2048^2 grid): no wasted re-reads.
  cells = 2048 * 2048
  assert table['fvm_explicit_2048'] <= 20 * cells
  assert table['spec_col_stage_2048'] <= 36 * cells
  assert table['spec_row_2048'] <= 20 * cells
