// Host entry to the double-word WENO5 of weno_exact.h (the same operations
// the PARITY kernels evaluate on the device), for tests on machines without
// a GPU.
#include <cstdint>

#include "../../include/gbls.h"
#include "weno_exact.h"

extern "C" int gbls_host_weno5_exact(int64_t n, const float* v, float* out, uint8_t* decided) {
    if (n < 0 || (n > 0 && (!v || !out || !decided))) return GBLS_ERR_INVALID_ARGUMENT;
    for (int64_t i = 0; i < n; ++i) {
        float r = 0.0f;
        const float* q = v + 5 * i;
        decided[i] = uint8_t(gbls::xw::weno5<float>(q[0], q[1], q[2], q[3], q[4], r) ? 1 : 0);
        out[i] = r;
    }
    return GBLS_OK;
}

// The sign that xw::weno5_sign certifies for each quintuple (+1: result
// >= 0, -1: result <= 0, 2: a zero, 0: undecided).
extern "C" int gbls_host_weno5_sign(int64_t n, const float* v, int8_t* sign) {
    if (n < 0 || (n > 0 && (!v || !sign))) return GBLS_ERR_INVALID_ARGUMENT;
    for (int64_t i = 0; i < n; ++i) {
        const float* q = v + 5 * i;
        sign[i] = int8_t(gbls::xw::weno5_sign(q[0], q[1], q[2], q[3], q[4]));
    }
    return GBLS_OK;
}

// weno5_sign_pair for n lines of six differences d[6i..6i+5]: the signs of
// the backward (d0..d4) and forward (d5..d1) operand sets.
extern "C" int gbls_host_weno5_sign_pair(int64_t n, const float* d, int8_t* sb, int8_t* sf) {
    if (n < 0 || (n > 0 && (!d || !sb || !sf))) return GBLS_ERR_INVALID_ARGUMENT;
    for (int64_t i = 0; i < n; ++i) {
        const float* q = d + 6 * i;
        int b = 0, f = 0;
        gbls::xw::weno5_sign_pair(q[0], q[1], q[2], q[3], q[4], q[5], b, f);
        sb[i] = int8_t(b);
        sf[i] = int8_t(f);
    }
    return GBLS_OK;
}
