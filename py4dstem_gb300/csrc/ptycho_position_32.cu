// Fused per-position kernels for the 32 x 32 region of interest (128 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES(32, 128)
