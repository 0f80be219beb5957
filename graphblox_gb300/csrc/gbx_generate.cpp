// Synthetic inputs (no reference counterpart: the reference reads edge lists
// from files). Counter-based generation: every edge draws from a stream keyed
// by (seed, edge index), so the output does not depend on the thread count or
// the host architecture.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "gbx.h"

namespace {

inline uint64_t mix64(uint64_t z) {
    // splitmix64 finaliser (Steele, Lea, Flood 2014)
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t stream_key(uint64_t seed, uint64_t index) {
    return mix64(seed * 0xD1B54A32D192ED03ull + 0x9E3779B97F4A7C15ull) ^ (index * 0x9E3779B97F4A7C15ull);
}

}  // namespace

extern "C" int gbx_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                                 uint64_t seed, uint32_t *src, uint32_t *dst) {
    if (!src || !dst || scale == 0 || scale > 30 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return GBX_ERR_INVALID;
    // quadrant thresholds on a 32-bit uniform draw
    const uint64_t two32 = 1ull << 32;
    const uint64_t ta = (uint64_t)(a * (double)two32);
    const uint64_t tab = (uint64_t)((a + b) * (double)two32);
    const uint64_t tabc = (uint64_t)((a + b + c) * (double)two32);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < (int64_t)num_edges; ++e) {
        uint64_t x = stream_key(seed, (uint64_t)e);
        uint32_t s = 0, d = 0;
        uint64_t bits = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            if ((l & 1u) == 0) {
                x += 0x9E3779B97F4A7C15ull;
                bits = mix64(x);
            }
            uint64_t r = (l & 1u) ? (bits >> 32) : (bits & 0xFFFFFFFFull);
            uint32_t bs, bd;
            if (r < ta) { bs = 0; bd = 0; }
            else if (r < tab) { bs = 0; bd = 1; }
            else if (r < tabc) { bs = 1; bd = 0; }
            else { bs = 1; bd = 1; }
            s = (s << 1) | bs;
            d = (d << 1) | bd;
        }
        src[e] = s;
        dst[e] = d;
    }
    return GBX_OK;
}

extern "C" int gbx_generate_values(uint64_t count, int kind, uint32_t lo, uint32_t hi, uint64_t seed,
                                   float *out) {
    if (!out || kind < 0 || kind > 3 || (kind == 0 && hi < lo)) return GBX_ERR_INVALID;
    const uint64_t span = (uint64_t)hi - lo + 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)count; ++i) {
        uint64_t h = mix64(stream_key(seed, (uint64_t)i) + 0x632BE59BD9B4E019ull);
        float v;
        switch (kind) {
        case 0: v = (float)(lo + (uint32_t)(h % span)); break;
        case 1: v = (float)((double)((h >> 40) + 1) / 16777216.0); break;             // (0, 1]
        case 2: v = (float)((double)(h >> 40) / 8388608.0 - 1.0); break;               // [-1, 1)
        default: {
            // lognormal(0, 1) by Box-Muller on two 26-bit uniforms in (0, 1)
            double u1 = ((double)(h >> 38) + 0.5) / 67108864.0;
            double u2 = ((double)((h >> 12) & 0x3FFFFFFull) + 0.5) / 67108864.0;
            double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            v = (float)std::exp(z);
        }
        }
        out[i] = v;
    }
    return GBX_OK;
}
