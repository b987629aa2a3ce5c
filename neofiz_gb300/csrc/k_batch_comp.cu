// k_batch_comp.cu -- the compensated batch form (NF_PRECISION_COMPENSATED): the persistent
// batched kernel with the FP32 nodal update and gather, instantiated here so that this
// translation unit alone is compiled with float multiply-add contraction, fast float division
// and square root and denormal flushing. None of them touches the FP64 and mixed forms
// (k_batch.cu), whose bits are fixed.
#include "nf_batch_kernels.cuh"

namespace nf {

// The compensated form's FP32 node state from the FP64 arrays (after the first assembly), and
// back (after a run, so reads and measurements see FP64 arrays).
__global__ void k_batch_comp_init(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const double2 x = d.X0[i], u = d.U[i], v = d.V[i], f = d.F[i];
    const float2 xr = ff_from(x.x), xz = ff_from(x.y), ur = ff_from(u.x), uz = ff_from(u.y);
    d.x0C[i] = make_float4(xr.x, xr.y, xz.x, xz.y);
    d.uC[i] = make_float4(ur.x, ur.y, uz.x, uz.y);
    d.vC[i] = make_float2((float)v.x, (float)v.y);
    d.fC[i] = make_float2((float)f.x, (float)f.y);
    d.mC[i] = make_float2((float)d.mass[i], (float)d.invMass[i]);
}

__global__ void k_batch_comp_sync(Dev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.N) return;
    const float4 u = d.uC[i];
    const float2 v = d.vC[i], f = d.fC[i];
    d.U[i] = make_double2((double)u.x + (double)u.y, (double)u.z + (double)u.w);
    d.V[i] = make_double2((double)v.x, (double)v.y);
    d.F[i] = make_double2((double)f.x, (double)f.y);
}

const void *comp_steps_kernel(const BatchShape &s) {
    if (s.stage) {
        if (s.threads == 32) return (const void *)k_batch_steps_comp<true, 32>;
        return s.threads == 128 ? (const void *)k_batch_steps_comp<true, 128>
                                : (const void *)k_batch_steps_comp<true, 256>;
    }
    if (s.threads == 32) return (const void *)k_batch_steps_comp<false, 32>;
    return s.threads == 128 ? (const void *)k_batch_steps_comp<false, 128>
                            : (const void *)k_batch_steps_comp<false, 256>;
}

void launch_batch_comp(const Dev &d, bool toFloat, cudaStream_t st) {
    if (d.N <= 0) return;
    if (toFloat) k_batch_comp_init<<<grid_for(d.N, 256), 256, 0, st>>>(d);
    else k_batch_comp_sync<<<grid_for(d.N, 256), 256, 0, st>>>(d);
}

}  // namespace nf
