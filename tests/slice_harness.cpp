// Host harness for the tensor-core slicing helpers (helios_gb300/csrc/hx_slice.h):
// reads "row_max_hex x_hex" lines, prints e = frexp exponent of the row maximum,
// the 3- and 5-digit splittings of x against that exponent, then 1 if the
// kernels' form of the splitting (slice_digits_fast, digit_value) gives the
// same digits and bf16 values for 3, 4, 5 and 7 digits, else 0.
#include <cmath>
#include <cstdio>

#include "hx_slice.h"

template <int S>
static bool same(double x, int e)
{
    int a[S], b[S];
    tc::slice_digits<S>(x, e, a);
    tc::slice_digits_fast<S>(x, e, b);
    for (int p = 0; p < S; ++p)
        if (a[p] != b[p] || tc::digit_value(b[p], p) != (float)std::ldexp((double)a[p], -8 * p)) return false;
    return true;
}

int main()
{
    double mx, x;
    while (scanf("%la %la", &mx, &x) == 2) {
        unsigned long long mb = tc::dbits(mx) & 0x7FFFFFFFFFFFFFFFull;
        int e = mb ? tc::exp_of_bits(mb) : 0;
        int s3[3], s5[5];
        tc::slice_digits<3>(x, e, s3);
        tc::slice_digits<5>(x, e, s5);
        const bool ok = same<3>(x, e) && same<4>(x, e) && same<5>(x, e) && same<7>(x, e);
        printf("%d %d %d %d %d %d %d %d %d %d\n", e, s3[0], s3[1], s3[2], s5[0], s5[1], s5[2], s5[3], s5[4], ok ? 1 : 0);
    }
    return 0;
}
