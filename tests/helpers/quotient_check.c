/* Exhaustive check of the kernel's per-segment quotient: for every
 * denominator d = len_path_2 - 1 in [1, D] and every span s in [1, d + 1],
 *     q0 = fl(s * r), r = fl(1/d);  e = fma(-q0, d, s);  q = fma(e, r, q0)
 * must equal the correctly rounded fl(s / d) the reference computes.
 * Prints the number of mismatches. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

int main(int argc, char **argv)
{
    int D = argc > 1 ? atoi(argv[1]) : 8192;
    long long bad = 0, n = 0;
    for (int d = 1; d <= D; d++) {
        volatile double dd = (double)d;
        double r = 1.0 / dd;
        for (int s = 1; s <= d + 1; s++) {
            double sd = (double)s;
            double q0 = sd * r;
            double e = fma(-q0, dd, sd);
            double q = fma(e, r, q0);
            double ref = sd / dd;
            n++;
            if (q != ref)
                bad++;
        }
    }
    printf("%lld %lld\n", n, bad);
    return 0;
}
