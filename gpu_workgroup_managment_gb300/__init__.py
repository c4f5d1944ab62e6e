"""GB300-native cooperative-kernel runtime: persistent graph kernels
synchronised by an inter-CTA barrier, behind the reference's scheduler_rt
host API (C-ABI in include/wgm.h, implemented by libwgm.so)."""
from . import graphs
from ._lib import WgmError
from .runtime import APPS, PersistentApp, Runtime, RunStats, default_config, solve

__all__ = ["graphs", "WgmError", "APPS", "PersistentApp", "Runtime", "RunStats",
           "default_config", "solve"]
