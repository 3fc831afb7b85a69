/* Stage and CFS-PML kernels of the iso medium (see cgfd_launch.cuh). */
#include "cgfd_media.cuh"
#define CGFD_MED MED_ISO
#define CGFD_MED_NAME iso
#include "cgfd_launch.cuh"

int cgfd_stage_smem_bytes(int med)
{
  return med == MED_VTI ? s3::Slot<MED_VTI>::SMEM_BYTES
       : med == MED_VIS ? s3::Slot<MED_VIS>::SMEM_BYTES
                        : s3::Slot<MED_ISO>::SMEM_BYTES;
}
