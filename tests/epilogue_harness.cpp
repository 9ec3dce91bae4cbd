// Host harness for the integer conversions of the tensor-core GEMM's
// epilogue (helios_gb300/csrc/hx_slice.h). Input lines:
//   "f hi_hex lo_hex k neg"  -> f2d_pow2(hi) + f2d_pow2(lo) (the epilogue's (hi + lo) 2^k): "1 value_hex"
//   "p x_hex k"              -> pow2_int(x, k):          "ok value_hex"
//   "c a_hex q"              -> class_count(a, q):       "n"
#include <cstdio>

#include "hx_slice.h"

int main()
{
    char op;
    while (scanf(" %c", &op) == 1) {
        if (op == 'f') {
            double hi, lo;
            int k;
            unsigned neg;
            if (scanf("%la %la %d %u", &hi, &lo, &k, &neg) != 4) return 1;
            const unsigned m = neg ? 0x80000000u : 0u;
            const double r = tc::f2d_pow2((float)hi, k, m) + tc::f2d_pow2((float)lo, k, m);
            printf("1 %a\n", r);
        } else if (op == 'p') {
            double x;
            int k;
            if (scanf("%la %d", &x, &k) != 2) return 1;
            bool ok = true;
            const double r = tc::pow2_int(x, k, ok);
            printf("%d %a\n", ok ? 1 : 0, r);
        } else if (op == 'c') {
            double a;
            int q;
            if (scanf("%la %d", &a, &q) != 2) return 1;
            printf("%d\n", tc::class_count((float)a, q));
        } else {
            return 1;
        }
    }
    return 0;
}
