/* Batched stage kernels of the vti medium (see cgfd_launch.cuh); the same
 * tile geometry as cgfd_launch_vti.cu. */
#define CGFD_TILE_ROWS 11
#include "cgfd_media.cuh"
#define CGFD_MED MED_VTI
#define CGFD_MED_NAME vti
#define CGFD_SINGLE 0
#define CGFD_BATCH 1
#include "cgfd_launch.cuh"
