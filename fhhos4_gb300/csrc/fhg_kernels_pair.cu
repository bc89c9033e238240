// The block-sparse kernels instantiated for FP32 pairs (dfl, fhg_pair.h): the V-cycle of FP64-class
// accuracy on the FP32 pipe (FHG_PREC_DF). A translation unit of its own so that it compiles in
// parallel with the float and double instantiations of fhg_kernels.cu.
#include "fhg_bsr_kernels.cuh"

namespace fhg {

template void launch_dots3<dfl>(long long, int, const dfl*, const dfl*, const dfl*, const dfl*, const dfl*, const dfl*,
                                double*, cudaStream_t);
template void launch_axpy<dfl>(long long, double, const dfl*, dfl*, cudaStream_t);
template void launch_lincomb<dfl>(long long, double, const dfl*, double, const dfl*, dfl*, cudaStream_t);
template void launch_spmv<dfl>(const BsrView<dfl>&, int, const dfl*, const dfl*, dfl*, cudaStream_t);
template void launch_gs<dfl>(const BsrView<dfl>&, int, int, const dfl*, long long, const dfl*, dfl*, cudaStream_t, int,
                             int, dfl);
template void launch_jacobi<dfl>(const BsrView<dfl>&, const dfl*, long long, dfl, const dfl*, const dfl*, dfl*,
                                 cudaStream_t);
template void launch_coarse<dfl>(int, const double*, const dfl*, dfl*, cudaStream_t);
template void launch_convert<dfl, double>(long long, const dfl*, double*, cudaStream_t);
template void launch_permute<dfl>(int, int, const int*, const dfl*, dfl*, bool, cudaStream_t);
template void launch_inject<dfl>(int, int, int, const int*, const dfl*, const dfl*, dfl*, bool, cudaStream_t);

}  // namespace fhg
