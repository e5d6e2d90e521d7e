// Wide node record access and the conservative quantiser, shared by the host
// builder (wide_build.cu) and the device kernels (k_wide.cu).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "device_common.cuh"
#include "wide.h"

namespace fcpwgb {

template<int W, int BITS> struct WideLayout {
    static constexpr int kHeader = wideHeaderBytes(BITS);
    static constexpr int kRefs = kHeader;
    static constexpr int kCnt = wideCntOffset(W, BITS);
    static constexpr int kBounds = wideBoundsOffset(W, BITS);
    static constexpr int kSize = wideNodeBytes(W, BITS);
    static constexpr int kBoundBytes = BITS / 8;
    static constexpr uint32_t kQMax = BITS == 8 ? 255u : 65535u;
};

FCPWGB_HD float exp2i(int e) {  // 2^e for e in [-126, 127]
#ifdef __CUDA_ARCH__
    return __int_as_float((e + 127) << 23);
#else
    uint32_t u = (uint32_t)(e + 127) << 23;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

FCPWGB_HD float fmaRn(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

// Writes header and bounds of a node record from W child boxes
// (lo/hi[c*3 + axis]); empty slots are marked by valid[c] == false. Returns
// false when a float box cannot be represented (non-finite input).
template<int W, int BITS>
FCPWGB_HD bool quantizeWideNode(const float *lo, const float *hi, const bool *valid, unsigned char *rec) {
    using L = WideLayout<W, BITS>;
    if (BITS == 32) {
        for (int a = 0; a < 3; a++)
            for (int c = 0; c < W; c++) {
                float l = valid[c] ? lo[c * 3 + a] : 0.0f, h = valid[c] ? hi[c * 3 + a] : 0.0f;
                std::memcpy(rec + L::kBounds + 4 * (a * W + c), &l, 4);
                std::memcpy(rec + L::kBounds + 4 * (3 * W + a * W + c), &h, 4);
            }
        return true;
    }
    int nValid = 0;
    for (int c = 0; c < W; c++) nValid += valid[c] ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        float o = 3.402823466e+38F, mx = -3.402823466e+38F;
        for (int c = 0; c < W; c++) {
            if (!valid[c]) continue;
            o = fminf(o, lo[c * 3 + a]);
            mx = fmaxf(mx, hi[c * 3 + a]);
        }
        if (nValid == 0) { o = 0.0f; mx = 0.0f; }
        if (!(o == o) || !(mx == mx) || fabsf(o) > 1e37f || fabsf(mx) > 1e37f) return false;
        double ext = (double)mx - (double)o;
        // smallest e with 2^e * qmax >= ext
        int e = -126;
        if (ext > 0.0) {
            int ex;
            (void)frexp(ext / (double)L::kQMax, &ex);  // ext/qmax = m * 2^ex, m in [0.5, 1)
            e = ex;
            if (e < -126) e = -126;
        }
        bool done = false;
        for (int attempt = 0; attempt < 4 && !done; attempt++, e++) {
            if (e > 127) return false;
            float s = exp2i(e);
            done = true;
            for (int c = 0; c < W && done; c++) {
                uint32_t ql = 0, qh = 0;
                if (valid[c]) {
                    double fl = floor(((double)lo[c * 3 + a] - (double)o) / (double)s);
                    double fh = ceil(((double)hi[c * 3 + a] - (double)o) / (double)s);
                    ql = fl < 0.0 ? 0u : (fl > (double)L::kQMax ? L::kQMax : (uint32_t)fl);
                    qh = fh < 0.0 ? 0u : (fh > (double)L::kQMax ? L::kQMax : (uint32_t)fh);
                    while (ql > 0 && fmaRn((float)ql, s, o) > lo[c * 3 + a]) ql--;
                    while (fmaRn((float)qh, s, o) < hi[c * 3 + a]) {
                        if (qh == L::kQMax) { done = false; break; }
                        qh++;
                    }
                    if (fmaRn((float)ql, s, o) > lo[c * 3 + a]) done = false;
                }
                if (BITS == 8) {
                    rec[L::kBounds + a * W + c] = (unsigned char)ql;
                    rec[L::kBounds + 3 * W + a * W + c] = (unsigned char)qh;
                } else {
                    uint16_t l16 = (uint16_t)ql, h16 = (uint16_t)qh;
                    std::memcpy(rec + L::kBounds + 2 * (a * W + c), &l16, 2);
                    std::memcpy(rec + L::kBounds + 2 * (3 * W + a * W + c), &h16, 2);
                }
            }
            if (done) {
                std::memcpy(rec + 4 * a, &o, 4);
                rec[12 + a] = (unsigned char)(e + 127);
            }
        }
        if (!done) return false;
    }
    rec[15] = (unsigned char)nValid;
    return true;
}

}  // namespace fcpwgb
