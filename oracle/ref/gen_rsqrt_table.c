/* Measures the x86 RSQRTPS approximation on this CPU and writes it as a table.
 *
 * The reference's AVX2 build computes sqrt(v) as v * rsqrt(v) (vector/avx.hh:412-415) and uses it
 * in the early-exit bound of sphere_environment_in_collision (collision/validity.hh:58).  On the
 * Intel CPUs measured so far the instruction's result depends only on the input's exponent parity
 * and the top 10 mantissa bits, scales exactly by powers of four, and returns +inf for zero and
 * subnormal inputs.  This program checks those three properties over every positive float and
 * then writes the 2048-entry table for inputs in [1, 4).  x86-64 only; test infrastructure.
 *
 *   gcc -O2 -mavx gen_rsqrt_table.c -o gen && ./gen out1.h out2.inc ...  */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float rsq(float x)
{
    return _mm_cvtss_f32(_mm_rsqrt_ss(_mm_set_ss(x)));
}

static uint32_t bits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

static float from_bits(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

int main(int argc, char **argv)
{
    float table[2048];
    for (uint32_t i = 0; i < 2048; ++i)
    {
        const uint32_t e = 127 + (i >> 10);           /* [1,2) then [2,4) */
        table[i] = rsq(from_bits((e << 23) | ((i & 1023u) << 13)));
    }
    /* verify the model over every positive normal float, and the special inputs */
    long bad = 0;
    for (uint32_t u = 0x00800000u; u < 0x7f800000u; ++u)
    {
        const float x = from_bits(u);
        const int E = (int)(u >> 23) - 127;
        const int odd = E & 1;
        const int k = (E - odd) / 2; /* x = 4^k * m, m in [1,4) */
        const uint32_t idx = ((uint32_t)odd << 10) | ((u >> 13) & 1023u);
        /* table[idx] * 2^-k, exact: scale the exponent field */
        const uint32_t tb = bits(table[idx]);
        const int te = (int)(tb >> 23) - k;
        float model;
        if (te <= 0)
            model = 0.0f; /* not reached for normal inputs */
        else
            model = from_bits(((uint32_t)te << 23) | (tb & 0x7fffffu));
        if (bits(model) != bits(rsq(x)))
            ++bad;
    }
    const float specials[] = {0.0f, 1e-45f, 1e-39f, 1.1754942e-38f};
    for (int i = 0; i < 4; ++i)
        if (bits(rsq(specials[i])) != 0x7f800000u)
            ++bad;
    if (bad)
    {
        fprintf(stderr, "rsqrt model mismatch on %ld inputs: this CPU does not fit the table model\n", bad);
        return 1;
    }
    for (int a = 1; a < argc; ++a)
    {
        FILE *f = fopen(argv[a], "w");
        if (!f)
            return 2;
        fprintf(f, "/* x86 RSQRTPS results for inputs in [1, 4), measured by oracle/ref/gen_rsqrt_table.c.\n"
                   " * Entry (odd << 10 | m10): input exponent 127 + odd, top 10 mantissa bits m10. */\n");
        for (int i = 0; i < 2048; ++i)
            fprintf(f, "0x%08xu,%s", bits(table[i]), (i % 8 == 7) ? "\n" : " ");
        fclose(f);
    }
    printf("rsqrt table verified over all positive normal floats; wrote %d file(s)\n", argc - 1);
    return 0;
}
