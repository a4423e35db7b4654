// Instantiates the sweep kernels for NF = 17 .. 24 (see boss_sweep_kernels.cuh).
#include "boss_sweep_kernels.cuh"

BOSS_SWEEP_RANGE(sweep_nf_c, 17)
