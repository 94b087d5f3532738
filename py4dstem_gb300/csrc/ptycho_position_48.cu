// Fused per-position kernels for the 48 x 48 region of interest (192 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES(48, 192)
