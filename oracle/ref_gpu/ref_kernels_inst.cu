/*
 * ref_kernels_inst.cu -- TEST INFRASTRUCTURE ONLY.
 *
 * Explicit instantiations of the reference's GCOO kernel templates, so that the
 * reference's own GPU code can be compiled into a device-only cubin for sm_103a
 * (oracle/Makefile, target `refgpu`, output oracle/_ref/ref_gcoo_sm103a.cubin)
 * and run on a GB300 next to this library on identical device buffers.
 *
 * The kernel file itself (src/gcoo_spdm_kernels.cu) and the tile constants
 * (src/constants.h) are included unmodified from the reference tree by the
 * build recipe; nothing of them is stored in this repository. The instances
 * are the ones the reference plugin launches (src/ShGCOOSpDM.cu:44-48,85-93,
 * 137-149: BS_OF_CAL = 512 for the conversion, BS and COLUMN_PER_GROUP from
 * constants.h for the multiply), plus the conversion for the other group
 * sizes the format allows (1, 2, 8, 16 rows per group).
 *
 * The host side (oracle/ref_gpu/ref_gpu_runner.c) finds the instances by
 * name in the loaded module and launches them with the reference's shapes.
 */
#include "constants.h"
#include "gcoo_spdm_kernels.cu"

#define REF_CONVERT_INSTANCES(CPG)                                                                      \
    template __global__ void cal_group_coo_format_nnz_kernel_cm<512, CPG>(float *, int, int, int *);     \
    template __global__ void convert_to_group_coo_format_kernel_cm<512, CPG>(float *, int, int, float *, \
                                                                             int *, int *, int *, int *);

REF_CONVERT_INSTANCES(1)
REF_CONVERT_INSTANCES(2)
REF_CONVERT_INSTANCES(4)
REF_CONVERT_INSTANCES(8)
REF_CONVERT_INSTANCES(16)

template __global__ void sparse_dense_groupcoo_mat_mul_kernel<BS, COLUMN_PER_GROUP>(float *, int *, int *, int *,
                                                                                    int *, int, int, float *, int,
                                                                                    int, float *);

/* The constants the cubin was built with, for the runner to check. */
extern "C" __global__ void ref_gcoo_constants(int *out)
{
    out[0] = COLUMN_PER_GROUP;
    out[1] = BS;
}
