// Host-side checks of the per-face march rules (no GPU): for random
// reflections, every face rule that can be an exit face of its leg marches in
// the octant of the leg's direction, and the field march's skip multiplier
// never exceeds 2^16 / qmax.  Prints "ok <cases>" or the first failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "anacor_internal.h"

using namespace anacor;

int main()
{
    std::mt19937_64 gen(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    const double F[9] = {0.98, 0.1, -0.05, -0.08, 0.97, 0.12, 0.06, -0.11, 0.99};
    const double axis[3] = {1.0, 0.0, 0.0}, xray[3] = {0.0, 0.0, -1.0};
    long long cases = 0;
    for (int it = 0; it < 20000; it++) {
        double s1[3] = {U(gen), U(gen), U(gen)};
        const double n = std::sqrt(s1[0] * s1[0] + s1[1] * s1[1] + s1[2] * s1[2]);
        if (n < 1e-3)
            continue;
        for (double &x : s1)
            x /= n;
        const double omega = (U(gen) + 1.0) * 3.141592653589793;
        ReflTable t;
        double rx[3], rs[3];
        if (setup_reflection(axis, omega, F, xray, s1, &t, rx, rs) != kOk)
            continue;
        for (int leg = 0; leg < 2; leg++) {
            const uint32_t sb = t.head[leg].sign_bits;
            const uint32_t oct = ((sb >> 5) & 1u) | ((sb >> 3) & 2u) | ((sb >> 1) & 4u);
            // face code -> (axis, max side): 1 x max, 6 x min, 5 y max, 4 y min, 3 z max, 2 z min
            const int faces[6][3] = {{1, 2, 1}, {6, 2, 0}, {5, 1, 1}, {4, 1, 0}, {3, 0, 1}, {2, 0, 0}};
            for (const auto &f : faces) {
                const int a = f[1];
                const bool toward = f[2] ? ((sb >> a) & 1u) : ((sb >> (3 + a)) & 1u);
                const FaceRule &R = t.rule[leg][f[0] - 1];
                if (!toward || R.status || !R.fast)
                    continue;
                cases++;
                if (R.octant != oct) {
                    std::printf("octant mismatch: refl %d leg %d face %d rule %u direction %u\n", it, leg, f[0],
                                (unsigned)R.octant, oct);
                    return 1;
                }
                const int s = R.count_axis, ia = s == 0 ? 1 : 0, ib = s == 2 ? 1 : 2;
                const double qmax = std::fmax(std::fabs(R.q[ia]), std::fabs(R.q[ib]));
                if (std::fabs(std::fabs(R.q[s]) - 1.0) != 0.0) {
                    std::printf("count axis ratio is not +-1: %g\n", R.q[s]);
                    return 1;
                }
                if (qmax > 0.0 && (double)R.skip_rq > 65536.0 / qmax) {
                    std::printf("skip multiplier too large: %u for qmax %.17g\n", R.skip_rq, qmax);
                    return 1;
                }
                // the largest skip from a field byte never leaves the proven box
                for (uint32_t d = 2; d <= 31; d++) {
                    const int n = std::min((int)d - 1, (int)(((d - 2u) * R.skip_rq) >> 16));
                    // box of half-width d - 1: n steps on the step axis, at most
                    // ceil(n qmax) + 1 on the others
                    if (n > 0 && std::ceil(n * qmax) > (double)(d - 2)) {
                        std::printf("skip %d from distance %u exceeds the box (qmax %.17g)\n", n, d, qmax);
                        return 1;
                    }
                }
            }
        }
    }
    std::printf("ok %lld\n", cases);
    return cases > 10000 ? 0 : 1;
}
