// Host build of the backprojector's stream-K partition (sk_split.h): for many
// (tiles, units per tile, CTAs) it checks that the CTA ranges cover every unit
// once, that sk_cta_of names the owner of every unit, and that every segment
// index a CTA derives for a tile is below sk_max_segments.  Prints the number
// of cases and of failures.
#include <cstdio>
#include <random>
#include <vector>

#include "../../ct_recon_extensions_gb300/csrc/sk_split.h"

using namespace ctr;

static int check(long long tiles, int nb, int sms)
{
    const long long U = tiles * nb;
    const int G = static_cast<int>(U < sms ? U : sms);
    std::vector<int> owner(U, -1);
    for (int c = 0; c < G; ++c)
        for (long long u = sk_unit_begin(c, G, U); u < sk_unit_begin(c + 1, G, U); ++u) {
            if (owner[u] != -1) return 1;
            owner[u] = c;
        }
    for (long long u = 0; u < U; ++u)
        if (owner[u] < 0 || sk_cta_of(u, G, U) != owner[u]) return 1;
    const int maxseg = sk_max_segments(tiles, nb, G);
    for (int c = 0; c < G; ++c) {
        const long long u0 = sk_unit_begin(c, G, U), u1 = sk_unit_begin(c + 1, G, U);
        for (long long t = u0 / nb; t * nb < u1; ++t) {
            const int seg = c - sk_cta_of(t * nb, G, U);
            if (seg < 0 || seg >= maxseg) return 1;
        }
    }
    return 0;
}

int main()
{
    std::mt19937 rng(3);
    int cases = 0, bad = 0;
    const int fixed[][3] = {{128, 23, 152}, {1, 3, 152}, {2, 3, 152}, {512, 23, 152}, {607, 72, 152},
                            {3, 2, 152}, {1, 2, 1}, {64, 72, 148}};
    for (auto& f : fixed) {
        bad += check(f[0], f[1], f[2]);
        ++cases;
    }
    for (int i = 0; i < 400; ++i) {
        const long long tiles = 1 + rng() % 700;
        const int nb = 2 + static_cast<int>(rng() % 130);
        const int sms[] = {152, 148, 7, 1};
        bad += check(tiles, nb, sms[rng() % 4]);
        ++cases;
    }
    std::printf("%d %d\n", cases, bad);
    return 0;
}
