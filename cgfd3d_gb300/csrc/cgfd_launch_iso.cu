/* Stage and CFS-PML kernels of the iso medium (see cgfd_launch.cuh). */
#define CGFD_TILE_ROWS 12
#include "cgfd_media.cuh"
#define CGFD_MED MED_ISO
#define CGFD_MED_NAME iso
#define CGFD_BATCH 0
#include "cgfd_launch.cuh"

