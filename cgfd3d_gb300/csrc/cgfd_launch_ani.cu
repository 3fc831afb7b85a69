/* Stage and CFS-PML kernels of the fully anisotropic medium (see
 * cgfd_launch.cuh); 8-row tiles: 21 constants per point in the stream
 * slots. */
#define CGFD_TILE_ROWS 8
#include "cgfd_media.cuh"
#define CGFD_MED MED_ANI
#define CGFD_MED_NAME ani
#define CGFD_BATCH 0
#include "cgfd_launch.cuh"
