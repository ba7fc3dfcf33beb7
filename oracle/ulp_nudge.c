/*
 * ulp_nudge.c -- TEST INFRASTRUCTURE ONLY: never linked into the product.
 *
 * The oracle (ocpx_oracle.c, which reproduces the reference's results bit for
 * bit on the golden fixtures) compiled with every exp, log, pow, acos and cos
 * result moved by one unit in the last place (or k units: oc_set_nudge_ulps),
 * up or down according to a seeded hash of the argument.  The reference's outputs depend on the
 * rounding of its C library's transcendental functions; running this build
 * on a fixture measures by how much, per output quantity.  The parity tests
 * bound a GPU result, whose transcendentals come from CUDA's math library
 * (documented maximum error 1-2 ulp per call, glibc's about 0.5 ulp), by that
 * measured sensitivity of the reference's own algorithm; two-ulp moves cover
 * the documented maximum of CUDA's pow, cos and acos.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

static uint64_t nudge_seed = 1;
static int nudge_ulps = 1;

void oc_set_nudge_seed(uint64_t seed) { nudge_seed = seed; }
void oc_set_nudge_ulps(int k) { nudge_ulps = k < 1 ? 1 : k; }

static double nudge(double y, double x)
{
    uint64_t b;
    memcpy(&b, &x, sizeof b);
    b ^= nudge_seed * 0xD1B54A32D192ED03ull;
    b ^= b >> 29;
    b *= 0x9E3779B97F4A7C15ull;
    b ^= b >> 32;
    const double to = (b & 1u) ? INFINITY : -INFINITY;
    for (int k = 0; k < nudge_ulps; k++) y = nextafter(y, to);
    return y;
}

static double nudged_exp(double x) { return nudge(exp(x), x); }
static double nudged_log(double x) { return nudge(log(x), x); }
static double nudged_pow(double x, double y) { return nudge(pow(x, y), x + 3.0 * y); }
static double nudged_acos(double x) { return nudge(acos(x), x); }
static double nudged_cos(double x) { return nudge(cos(x), x); }

#define exp nudged_exp
#define log nudged_log
#define pow nudged_pow
#define acos nudged_acos
#define cos nudged_cos
#include "ocpx_oracle.c"
