// Galactic-binary waveform samples on the device, shared by the waveform
// kernel (flr_waveform.cu, waveforms written to memory) and the fused kernel
// (waveforms generated straight into its staged input window).
//
// Two models (GbParams::model), evaluated in FP64 with CUDA's double sincos
// (a few ulp from the host generators of fastlisaresponse_gb300.waveforms):
//   0  the benchmark configurations' binary (waveforms.gb_waveform):
//        Phi = phi0 + 2 pi (f t + fdot t^2 / 2),
//        hp0 = A (1 + cos^2 iota) cos Phi,  hc0 = -2 A cos iota sin Phi;
//   1  the reference test-suite's GBWave (tests/test_fastlisaresponse.py:34-63
//      of the reference; waveforms.GBWave): third-order phase with
//      fddot = 11/3 fdot^2 / f and phase origin -phi0,
//        Phi = 2 pi (f t + fdot t^2 / 2 + fddot t^3 / 6) - phi0,
//        hp0 = -cos Phi A (1 + cos^2 iota),  hc0 = -sin Phi 2 A cos iota;
// both rotated by the polarisation angle: hp = hp0 cos 2psi - hc0 sin 2psi,
// hc = hp0 sin 2psi + hc0 cos 2psi.
#pragma once

#include <cuda_runtime.h>

#include "flr_fused.h"

namespace flr {

struct GbCoefs {
    double amp_p, amp_c, c2, s2, f, half_fdot, sixth_fddot, phi0;
    int model;
};

__device__ __forceinline__ GbCoefs gb_coefs(const GbParams &p) {
    GbCoefs c;
    const double cosi = cos(p.iota);
    c.model = p.model;
    if (p.model == 1) {
        c.amp_p = p.A * (1.0 + cosi * cosi);
        c.amp_c = 2.0 * p.A * cosi;
        c.sixth_fddot = (1.0 / 6.0) * (11.0 / 3.0 * (p.fdot * p.fdot) / p.f);
    } else {
        c.amp_p = p.A * (1.0 + cosi * cosi);
        c.amp_c = -2.0 * p.A * cosi;
        c.sixth_fddot = 0.0;
    }
    sincos(2.0 * p.psi, &c.s2, &c.c2);
    c.f = p.f;
    c.half_fdot = 0.5 * p.fdot;
    c.phi0 = p.phi0;
    return c;
}

// h(t) = hp + i hc
__device__ __forceinline__ double2 gb_sample(const GbCoefs &c, double t) {
    double phase, sp, cp, hp0, hc0;
    if (c.model == 1) {
        phase = 6.283185307179586 * (c.f * t + c.half_fdot * (t * t) + c.sixth_fddot * (t * t * t)) -
                c.phi0;
        sincos(phase, &sp, &cp);
        hp0 = -cp * c.amp_p;
        hc0 = -sp * c.amp_c;
    } else {
        phase = c.phi0 + 6.283185307179586 * (c.f * t + c.half_fdot * t * t);
        sincos(phase, &sp, &cp);
        hp0 = c.amp_p * cp;
        hc0 = c.amp_c * sp;
    }
    return make_double2(hp0 * c.c2 - hc0 * c.s2, hp0 * c.s2 + hc0 * c.c2);
}

// The input of a source as the fused kernel reads it outside its staged
// window: the stored waveform h, or (h == NULL) the source's generator
// evaluated at t0 + k dt (its coefficients recomputed per call: such reads
// are rare).
struct HSrc {
    const double2 *h;
    const GbParams *g;
    double t0, dt;
    __device__ __forceinline__ double2 operator[](long k) const {
        if (h) return __ldg(h + k);
        return gb_sample(gb_coefs(*g), t0 + (double)k * dt);
    }
};

}  // namespace flr
