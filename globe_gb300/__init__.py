"""GB300-native GLOBE: the longitudinal genomic mixed-model solve of
ahmadazim/GLOBE (runPCGsolver / runAIREML) on one GPU.

The compute path is libglobe_gb300.so (hand-written sm_103a CUDA behind the C
ABI in include/globe.h); this package is its host-side binding.
"""
from ._lib import (GlobeError, MODEL_FULL, MODEL_NO_TIME, PREC_FP64, PREC_MIXED, RULE_AIREML, RULE_PCGSOLVER,
                   X0_GIVEN, X0_PRECOND, X0_ZERO)
from .api import (Context, as_float_vc, build_grm, read_bed, read_grm, read_records, read_records_no_time, read_vector,
                  run_aireml, run_pcg_solver, save_vector, trust_region_step, trust_region_step_no_time, write_grm)

__all__ = ["Context", "GlobeError", "MODEL_FULL", "MODEL_NO_TIME", "PREC_FP64", "PREC_MIXED", "RULE_AIREML",
           "RULE_PCGSOLVER", "X0_GIVEN", "X0_PRECOND", "X0_ZERO", "as_float_vc", "build_grm", "read_bed", "read_grm",
           "read_records", "read_records_no_time", "read_vector", "run_aireml", "run_pcg_solver", "save_vector",
           "trust_region_step", "trust_region_step_no_time", "write_grm"]
