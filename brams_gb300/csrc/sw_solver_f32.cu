// The fp32 instantiation of the RRTMG_SW column kernel (sw_kernel.cuh): gas
// optics, cloud optics and the two-stream solution in fp32 (with fused
// multiply-adds), fp64 for the layer coefficients, the flux accumulation over
// g-points and the heating rates.  Its table directory is this unit's own copy.
#include "sw_kernel.cuh"

cudaError_t gb_sw_set_tab_f32(const void* tab) { return gbsw::sw_set_tab(*static_cast<const gbsw::SwTab*>(tab)); }

cudaError_t gb_sw_launch_f32(const SwArgs& a, const float* d_tables, float* scratch, long long slots,
                             cudaStream_t stream) {
  return gbsw::sw_launch_t<float, SW_MINB_F32>(a, d_tables, scratch, slots, stream);
}
