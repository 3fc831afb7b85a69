/* Stage and CFS-PML kernels of the vti medium (see cgfd_launch.cuh). */
#define CGFD_TILE_ROWS 11
#include "cgfd_media.cuh"
#define CGFD_MED MED_VTI
#define CGFD_MED_NAME vti
#define CGFD_BATCH 0
#include "cgfd_launch.cuh"
