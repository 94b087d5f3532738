// Fused per-position kernels for the 96 x 128 region of interest (768 threads
// per block); the templates are in ptycho_position.cuh.
#include "ptycho_position.cuh"

PTY_POSITION_INSTANCES_XY(96, 128, 96x128, 768)
