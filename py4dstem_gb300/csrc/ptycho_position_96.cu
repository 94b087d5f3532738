// Fused per-position kernels for the 96 x 96 region of interest (384 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES(96, 384)
