// Host driver for tests/test_ozaki_fixed.py: evaluates the integer arithmetic of the tensor-core
// Cholesky (librpa_gb300/csrc/ozaki_fixed.h) on the cases read from stdin, one per line:
//   F w e0          -> fixed_to_double(w, e0) as the hex bit pattern
//   S xbits mbits   -> the 8 slice digits of entry xbits in a row whose maximum is mbits
//   C u0 u1 u2 u3   -> combine_groups(u0, u1, u2, u3)
#include <cinttypes>
#include <cstdio>
#include <cstring>

#include "ozaki_fixed.h"

int main()
{
    char op;
    while (std::scanf(" %c", &op) == 1)
    {
        if (op == 'F')
        {
            long long w;
            int e0;
            if (std::scanf("%lld %d", &w, &e0) != 2) return 1;
            const double d = gb::ozaki::fixed_to_double(w, e0);
            unsigned long long b;
            std::memcpy(&b, &d, sizeof b);
            std::printf("%016llx\n", b);
        }
        else if (op == 'S')
        {
            unsigned long long x, m;
            if (std::scanf("%llx %llx", &x, &m) != 2) return 1;
            int dig[gb::ozaki::OZ_SLICES];
            const int e = gb::ozaki::row_exponent(m);
            gb::ozaki::slice_digits(x, e, (m >> 52) != 0, dig);
            std::printf("%d", e);
            for (int p = 0; p < gb::ozaki::OZ_SLICES; ++p) std::printf(" %d", dig[p]);
            std::printf("\n");
        }
        else if (op == 'C')
        {
            int u[4];
            if (std::scanf("%d %d %d %d", &u[0], &u[1], &u[2], &u[3]) != 4) return 1;
            std::printf("%lld\n", gb::ozaki::combine_groups(u[0], u[1], u[2], u[3]));
        }
        else
            return 1;
    }
    return 0;
}
