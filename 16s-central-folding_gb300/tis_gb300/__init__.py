"""GB300 (sm_103a) TIS-RNA Langevin engine: Python binding of the C ABI.

from tis_gb300 import System, Engine
    sys = System.load(pdb, bonds, stacks, maxikey, T=0.615, c_mg=0.005, c_k=0.05, seed=1)
    eng = Engine([sys], precision=0)
    eng.step(1000); eng.sync()
"""
from .api import (ENERGY_NAMES, N_PARAMS, NOISE_OFF, NOISE_REFERENCE, PARAM_NAMES, PREC_FP64, PREC_MIXED, STATE_NAMES,
                  TERM_BONDED, TERM_HB, TERM_LR, TERM_SR, TERM_STACK, Engine, System, TisError, autotune, contact_concentration,
                  lib,
                  read_last_frame)

__all__ = ["System", "Engine", "TisError", "lib", "STATE_NAMES", "ENERGY_NAMES", "TERM_SR", "TERM_LR",
           "TERM_BONDED", "TERM_STACK", "TERM_HB", "PREC_MIXED", "PREC_FP64", "NOISE_REFERENCE", "NOISE_OFF",
           "read_last_frame", "PARAM_NAMES", "N_PARAMS", "autotune", "contact_concentration"]
