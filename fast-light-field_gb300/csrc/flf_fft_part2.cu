// Explicit instantiations of the size-specialised transforms for
// F in {8, 12, 24, 30, 54, 60, 84, 98, 126, 144}.
// The sizes are spread over several translation units so that they compile in parallel.
#include "flf_fft.cuh"

namespace flf {
namespace sfft {

FLF_SFFT_DEFINE_LAUNCHERS

template cudaError_t rfft2_sized<8>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<8>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<12>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<12>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<24>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<24>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<30>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<30>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<54>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<54>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<60>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<60>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<84>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<84>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<98>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<98>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<126>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<126>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<144>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<144>(const Irfft2Params &, cudaStream_t);

}  // namespace sfft
}  // namespace flf
