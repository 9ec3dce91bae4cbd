// Host harness for the amplitude layout conversions (helios_gb300/csrc/hx_layout.h):
// for each "o v" line, fills the column-major t1(o, v) and t2(o, o, v, v) with
// their own element numbers, converts them to the engine's layouts and prints
// the converted t1 and t2 (one number per line, engine order), then 1 if
// converting back gives the column-major arrays again, else 0.
#include <cstdio>
#include <vector>

#include "hx_layout.h"

int main()
{
    int o, v;
    while (scanf("%d %d", &o, &v) == 2) {
        const size_t ov = (size_t)o * v, n2 = ov * ov;
        std::vector<double> f1(ov), f2(n2), e1(ov), e2(n2), b1(ov, -1.0), b2(n2, -1.0);
        for (size_t k = 0; k < ov; ++k) f1[k] = (double)k;
        for (size_t k = 0; k < n2; ++k) f2[k] = (double)k;
        hx::t1_to_engine(f1.data(), e1.data(), o, v);
        hx::t2_to_engine(f2.data(), e2.data(), o, v);
        for (size_t k = 0; k < ov; ++k) printf("%.0f\n", e1[k]);
        for (size_t k = 0; k < n2; ++k) printf("%.0f\n", e2[k]);
        hx::t1_from_engine(e1.data(), b1.data(), o, v);
        hx::t2_from_engine(e2.data(), b2.data(), o, v);
        printf("%d\n", (b1 == f1 && b2 == f2) ? 1 : 0);
    }
    return 0;
}
