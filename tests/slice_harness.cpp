// Host harness for the tensor-core slicing helpers (helios_gb300/csrc/hx_slice.h):
// reads "row_max_hex x_hex" lines, prints e = frexp exponent of the row maximum
// and the 3- and 5-digit splittings of x against that exponent.
#include <cstdio>

#include "hx_slice.h"

int main()
{
    double mx, x;
    while (scanf("%la %la", &mx, &x) == 2) {
        unsigned long long mb = tc::dbits(mx) & 0x7FFFFFFFFFFFFFFFull;
        int e = mb ? tc::exp_of_bits(mb) : 0;
        int s3[3], s5[5];
        tc::slice_digits<3>(x, e, s3);
        tc::slice_digits<5>(x, e, s5);
        printf("%d %d %d %d %d %d %d %d %d\n", e, s3[0], s3[1], s3[2], s5[0], s5[1], s5[2], s5[3], s5[4]);
    }
    return 0;
}
