// Fused per-position kernels for the 64 x 64 region of interest (256 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES(64, 256)
