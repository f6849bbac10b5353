"""wavi_gb300 — GB300 (sm_103a) backend for WAVI.jl's velocity solve.

The package directory is ``wavi.jl_gb300/``; it is imported under the module name ``wavi_gb300``
(see ``__graft_entry__.load_package``).  Layout:

  csrc/         CUDA kernels (kernels.cuh) and the C ABI (wavi_gpu.cu) -> _build/libwavi_gpu.so
  abi.py        ctypes mirror of include/wavi_gpu.h
  gpu.py        VelocitySolver: one wavi_ctx per grid; host (e2e) and device entry points
  config.py     Grid / Params / SolverParams / TimesteppingParams / InitialConditions mirrors
  model.py      Model, update_state!, Simulation, run_simulation! with the GPU velocity solve plugged in
  ensemble.py   ensembles of independent domains solved at once, and their launch autotuner
  autograd.py   the adjoint behind a torch.autograd.Function
  misfit.py     the speed misfit (the adjoint workload's objective) and its velocity gradient
  schwarz.py    SharedMemorySpec's restricted additive Schwarz decomposition and sweeps
  io.py         file formats: the MITgcm velocity dump, JLD2 read/write, output files, their NetCDF merge
  synthetic.py  seeded synthetic geometries: the benchmark channels, small test cases, the iceberg
  build.py      nvcc build of the library
"""
from . import abi, config, synthetic  # noqa: F401
from .config import Grid, InitialConditions, OutputParams, Params, SolverParams, TimesteppingParams  # noqa: F401


def __getattr__(name):
    # the GPU-facing modules load libwavi_gpu.so lazily, so config-only users need no GPU
    if name in ("gpu", "model", "build"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
