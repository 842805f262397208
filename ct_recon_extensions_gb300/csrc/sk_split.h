// Stream-K partition of a launch's work units over its CTAs, shared by the
// backprojector's device code and host set-up (and built for the host by
// tests/cpp/sk_split_check.cc): CTA c of G owns units [c*U/G, (c+1)*U/G).
#pragma once

#if defined(__CUDACC__)
#define CTR_SK_HD __host__ __device__ __forceinline__
#else
#define CTR_SK_HD inline
#endif

namespace ctr {

// First unit of CTA c.
CTR_SK_HD long long sk_unit_begin(int c, int G, long long U) { return static_cast<long long>(c) * U / G; }

// The CTA whose range holds unit u: the largest c with c*U/G <= u, i.e.
// c*U < (u+1)*G.
CTR_SK_HD int sk_cta_of(long long u, int G, long long U)
{
    const long long c = ((u + 1) * G - 1) / U;
    return static_cast<int>(c < G - 1 ? c : G - 1);
}

// Most CTAs that share one tile of nb units.
CTR_SK_HD int sk_max_segments(long long tiles, int nb, int G)
{
    const long long U = tiles * nb;
    int m = 1;
    for (long long t = 0; t < tiles; ++t) {
        const int s = sk_cta_of(t * nb + nb - 1, G, U) - sk_cta_of(t * nb, G, U) + 1;
        m = s > m ? s : m;
    }
    return m;
}

}  // namespace ctr
