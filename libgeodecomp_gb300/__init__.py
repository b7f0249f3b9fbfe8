"""GB300-native cell-update hot path of LibGeoDecomp (host side in Python).

Modules:
  lgd              ctypes binding of the C ABI (include/lgd_*.h) in
                   liblgd_gb300.so: structured grids, SELL-C-sigma grids,
                   D3Q19 ensembles; raises if the library is not built
  build            compiles liblgd_gb300.so for sm_103a (nvcc, in-tree)
  workloads        seeded synthetic inputs of the benchmark configurations
  slabs            slab decomposition of structured grids over ranks
  sell_shards      row-block decomposition of SELL-C-sigma grids over ranks
  surrogate        the learned surrogate: network, training, judge
  surrogate_slabs  the surrogate's inference with its judge on z-slabs

The C++ drop-in for CUDASimulator<CELL> is header-only:
include/libgeodecomp_gb300/gb300simulator.h (with gb300cell.cuh for a
cell's own update() on the device and gb300stepper.h for one rank's slab).
"""
