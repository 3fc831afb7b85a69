/*
 * cgfd3d_dropin.h -- what the drop-in library (libcgfd3d_dropin.so, built
 * from cgfd3d_gb300/csrc/dropin/drv_rk_curv_col_gpu.c) exports beside
 * drv_rk_curv_col_allstep itself, whose prototype is the reference's
 * (forward/drv_rk_curv_col.h:17-37).
 *
 * The reference's time loop returns void and ends the process on errors
 * (MPI_Abort or exit, e.g. forward/drv_rk_curv_col.c:155-157), and so does
 * the drop-in: a device error, a bounded device wait that ran out, a
 * non-finite wavefield at a qc check step, or an unsupported configuration
 * prints a message to stderr and aborts.  The code of that failure stays
 * readable for a handler that runs at exit.
 */
#ifndef CGFD3D_DROPIN_H
#define CGFD3D_DROPIN_H

#ifdef __cplusplus
extern "C" {
#endif

/* CGFD_* code (include/cgfd3d_gpu.h) of the failure that ended the last
 * drv_rk_curv_col_allstep call: CGFD_EINVAL for unsupported or invalid
 * input, CGFD_ECUDA for a device error or wait timeout, CGFD_ENOMEM,
 * CGFD_ENONFINITE for the qc finiteness check; 0 while no call failed. */
int cgfd_gpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
