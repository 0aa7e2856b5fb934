// Explicit instantiations of the size-specialised transforms for
// F in {4, 10, 28, 32, 50, 56, 90, 96, 112, 160}.
// The sizes are spread over several translation units so that they compile in parallel.
#include "flf_fft.cuh"

namespace flf {
namespace sfft {

FLF_SFFT_DEFINE_LAUNCHERS

template cudaError_t rfft2_sized<4>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<4>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<10>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<10>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<28>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<28>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<32>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<32>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<50>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<50>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<56>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<56>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<90>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<90>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<96>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<96>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<112>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<112>(const Irfft2Params &, cudaStream_t);
template cudaError_t rfft2_sized<160>(const Rfft2Params &, cudaStream_t);
template cudaError_t irfft2_sized<160>(const Irfft2Params &, cudaStream_t);

}  // namespace sfft
}  // namespace flf
