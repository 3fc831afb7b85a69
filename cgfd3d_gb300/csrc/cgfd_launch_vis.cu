/* Stage and CFS-PML kernels of the vis medium (see cgfd_launch.cuh). */
#define CGFD_TILE_ROWS 8
#include "cgfd_media.cuh"
#define CGFD_MED MED_VIS
#define CGFD_MED_NAME vis
#define CGFD_BATCH 0
#include "cgfd_launch.cuh"
