// oracle/ref_kernels.cu -- TEST INFRASTRUCTURE: compiles the reference's own
// kernel sources, where they lie, into one cubin for oracle/ref_runner.cpp.
//
// The reference source is included unchanged (-I points at the reference
// tree; nothing of it is copied here).  tcfftCreate instantiates only the
// Volta fragment-map kernels (tcfft_half.cu:1244-1248; 2D
// tcfft_half_2d.cu:1160-1165); the sm_80 fragment-map variants ("_A100",
// tcfft_half.cu:164,393,702,886,1098; 2D tcfft_half_2d.cu:163,384,655,839,1049)
// are templates nothing instantiates, so they are instantiated below with the
// same <CONT_SIZE, NUM_WARP> arguments tcfftCreate gives their Volta twins.
#if TCFFT_REF_2D
#include "tcfft_half_2d.cu"
#else
#include "tcfft_half.cu"
#endif

template __global__ void layer_256_0_A100<32, 8>(half2*, half*, half*);
template __global__ void layer_512_0_A100<16, 8>(half2*, half*, half*);
template __global__ void layer_1024_0_A100<8, 8>(half2*, half*, half*);
template __global__ void layer_256_1_A100<32, 8>(int, half2*, half*, half*);
template __global__ void layer_512_1_A100<16, 8>(int, half2*, half*, half*);
