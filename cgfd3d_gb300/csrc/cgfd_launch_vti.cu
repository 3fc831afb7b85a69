/* Stage and CFS-PML kernels of the vti medium (see cgfd_launch.cuh). */
#include "cgfd_media.cuh"
#define CGFD_MED MED_VTI
#define CGFD_MED_NAME vti
#include "cgfd_launch.cuh"
