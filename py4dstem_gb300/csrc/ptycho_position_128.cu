// Fused per-position kernels for the 128 x 128 region of interest (1024 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES(128, 1024)
