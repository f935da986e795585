// Test infrastructure: build shim for compiling the reference's CPU branch.
//
// The reference's LISAResponse.cu includes "cuda_complex.hpp" from the
// lisaanalysistools package (not present in this environment).  The response
// code only needs a two-double complex value with real()/imag() accessors and
// the layout of std::complex<double> (the Python side hands it complex128
// buffers, binding_flr.hpp:133-141).  This header supplies exactly that, plus
// the host-side spellings of the CUDA portability macros the reference uses.
#ifndef ORACLE_REF_SHIM_CUDA_COMPLEX_HPP
#define ORACLE_REF_SHIM_CUDA_COMPLEX_HPP

#include <cmath>
#include <cstdio>
#include <stdexcept>

#ifndef CUDA_CALLABLE_MEMBER
#define CUDA_CALLABLE_MEMBER
#endif
#ifndef CUDA_KERNEL
#define CUDA_KERNEL
#endif
#ifndef CUDA_SHARED
#define CUDA_SHARED
#endif
#ifndef CUDA_SYNC_THREADS
#define CUDA_SYNC_THREADS
#endif
#ifndef CUDA_DEVICE
#define CUDA_DEVICE
#endif
#ifndef gpuErrchk
#define gpuErrchk(x) (x)
#endif

namespace gcmplx {

template <typename T>
class complex {
  public:
    complex() : re_(0), im_(0) {}
    complex(T re, T im = T(0)) : re_(re), im_(im) {}
    T real() const { return re_; }
    T imag() const { return im_; }

  private:
    T re_;
    T im_;
};

}  // namespace gcmplx

#endif
