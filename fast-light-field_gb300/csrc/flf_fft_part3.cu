// Explicit instantiations of the size-specialised transforms for
// F in {6, 14, 18, 40, 42, 70, 72, 108, 128, 140}.
// The sizes are spread over several translation units so that they compile in parallel.
#include "flf_fft.cuh"

namespace flf {
namespace sfft {

FLF_SFFT_DEFINE_LAUNCHERS

template cudaError_t rfft2_sized<6>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<6>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<14>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<14>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<18>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<18>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<40>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<40>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<42>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<42>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<70>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<70>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<72>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<72>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<108>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<108>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<128>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<128>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<140>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<140>(const Irfft2Params &, cudaStream_t);

}  // namespace sfft
}  // namespace flf
