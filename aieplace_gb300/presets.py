"""Workload presets of the seeded synthetic netlists (data only, no imports,
so CPU-only callers can read them without the product library).

  c0        576 unit cells on a 24x24 site die, 640 nets (70/20/10% 2/3/4-pin,
            uniform pins), 24 IO pads, 32x32 bins, target density 1.0
  c1        200k cells (width LogNormal(ln 2, 0.5), height 1 row), 2% fixed
            macros, 210k nets (65% 2, 20% 3, 10% 4-10, 5% 11-64 pins, 80%
            pins within a 64-node window), 512x512 bins, target density 0.7
  c2        2M cells, 1% macros, 2.1M nets, 1024x1024 bins, target density 0.8
  c1_small  / c2_small: the same distributions at 1/10 and 1/100 scale for tests
"""

PRESETS = {
    "c0": dict(num_cells=576, num_nets=640, num_macros=0, num_pads=24, unit_cells=1, degree_mix=0,
               locality=0.0, window=64, target_density=1.0, die_side=24.0, bins=32),
    "c1": dict(num_cells=200_000, num_nets=210_000, num_macros=4_000, num_pads=0, unit_cells=0,
               degree_mix=1, locality=0.8, window=64, target_density=0.7, die_side=0.0, bins=512),
    "c2": dict(num_cells=2_000_000, num_nets=2_100_000, num_macros=20_000, num_pads=0, unit_cells=0,
               degree_mix=1, locality=0.8, window=64, target_density=0.8, die_side=0.0, bins=1024),
    "c1_small": dict(num_cells=20_000, num_nets=21_000, num_macros=400, num_pads=0, unit_cells=0,
                     degree_mix=1, locality=0.8, window=64, target_density=0.7, die_side=0.0, bins=128),
    "c2_small": dict(num_cells=200_000, num_nets=210_000, num_macros=2_000, num_pads=0, unit_cells=0,
                     degree_mix=1, locality=0.8, window=64, target_density=0.8, die_side=0.0, bins=512),
}
