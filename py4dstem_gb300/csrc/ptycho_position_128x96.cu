// Fused per-position kernels for the 128 x 96 region of interest (768 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES_XY(128, 96, 128x96, 768)
