/* Batched stage kernels of the iso medium (see cgfd_launch.cuh); the same
 * tile geometry as cgfd_launch_iso.cu. */
#define CGFD_TILE_ROWS 12
#include "cgfd_media.cuh"
#define CGFD_MED MED_ISO
#define CGFD_MED_NAME iso
#define CGFD_SINGLE 0
#define CGFD_BATCH 1
#include "cgfd_launch.cuh"
