// Explicit instantiations of the size-specialised transforms for
// F in {2, 16, 20, 36, 48, 64, 80, 100, 120, 150}.
// The sizes are spread over several translation units so that they compile in parallel.
#include "flf_fft.cuh"

namespace flf {
namespace sfft {

FLF_SFFT_DEFINE_LAUNCHERS

template cudaError_t rfft2_sized<2>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<2>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<16>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<16>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<20>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<20>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<36>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<36>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<48>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<48>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<64>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<64>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<80>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<80>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<100>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<100>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<120>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<120>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<150>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<150>(const Irfft2Params &, cudaStream_t);

}  // namespace sfft
}  // namespace flf
