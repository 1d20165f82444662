"""GB300-native EMPEROR sampling hot path.

The batched Keplerian radial-velocity log-posterior that EMPEROR's
parallel-tempering engine evaluates for every walker at every temperature,
the affine-invariant stretch move and the temperature swaps, resident on one
GPU and reached through the C ABI of ``include/emp_gpu.h``
(``_lib/libemp_gpu.so``).

User surface (same names as EMPEROR):
    ``Simulation``  -- load_data / set_engine('reddemcee') / engine_config /
                       add_condition / autorun
    ``PTSampler``   -- reddemcee-compatible sampler on the GPU
"""
from .data import RVData, load_rv_folder, load_target, preprocess_instruments
from .model import (AccelerationBlock, JitterBlock, KeplerianBlock, MOAVBlock, OffsetBlock,
                    Parameter, Parameter_Block, ReddModel, SmartSetter)

__version__ = '0.1.0'


def __getattr__(name):
    # torch-dependent parts load lazily so that host-only imports stay light
    if name in ('PTSampler', 'Context', 'PTState', 'default_betas'):
        from . import engine
        return getattr(engine, name)
    if name == 'Simulation':
        from .simulation import Simulation
        return Simulation
    raise AttributeError(name)
