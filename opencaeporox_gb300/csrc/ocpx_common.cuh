// Shared device-side definitions for the FIM Newton-step kernels:
// model parameter blocks, table interpolation, small helpers.
//
// Every physics routine is written as an OCPX_HD (host+device) inline
// function operating on one cell, so kernels stay thin wrappers that map
// threads (or warps) to cells / rows / connections.
#pragma once

#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define OCPX_HD __host__ __device__ __forceinline__
#define OCPX_D __device__ __forceinline__
// large per-cell routines are kept out of line: they are called from many
// places in the flash, and inlining every call site multiplies code size and
// compile time without saving FP64 work
#define OCPX_HD_NOINLINE __host__ __device__ __noinline__
#else
#define OCPX_HD inline
#define OCPX_D inline
#define OCPX_HD_NOINLINE inline
#endif

namespace ocpx {

// ---------------------------------------------------------------- limits --
constexpr int NP = 3;            // phases: oil, gas, water (index 0,1,2)
constexpr int NC_MAX = 12;       // hydrocarbon components in the EoS (compositional)
constexpr int NCT_MAX = NC_MAX + 1;  // components incl. water
constexpr int TAB_ROWS_MAX = 64; // rows of any PVT / saturation table
constexpr int FLASH_CTRL_N = 13;

// reference constants (include/OCPConst.hpp:30-32, include/OCPEoS.hpp:111-112)
constexpr double TINY = 1E-8;
constexpr double PI_REF = 3.141592653;
constexpr double DELTA1 = 2.41421356237;
constexpr double DELTA2 = -0.41421356237;

// per-cell status bits reported by the kernels
enum : uint32_t {
    ST_OK = 0,
    ST_SPLIT_NONCONV = 1u << 0,   // phase split ended without NR convergence
    ST_STAB_NONCONV = 1u << 1,    // stability SSM/NR hit its iteration cap
    ST_SINGULAR = 1u << 2,        // zero pivot in a dense solve
    ST_NONFINITE = 1u << 3,       // NaN/Inf in the flash outputs
    ST_NEG_P = 1u << 4,           // negative pressure after the Newton update
    ST_NEG_NI = 1u << 5,          // negative moles beyond the clamp rule
    ST_ITER_CAP = 1u << 6,        // device-side iteration cap reached (watchdog)
};

// ----------------------------------------------------------------- table --
// Column-major table: col c, row r at data[c * nrow + r] (OCPTable::data[c][r]).
struct Table {
    int nrow;
    int ncol;
    double data[6 * TAB_ROWS_MAX];
};

// OCPTable::Eval_All with slopes (src/OCPTable.cpp:26-64): linear
// interpolation in column j; outside the range the end row is returned with
// zero slope.  The reference keeps a search hint between calls; the located
// interval does not depend on it, so the lookup here is stateless.
OCPX_HD int table_interval(const Table& t, int j, double val)
{
    const double* x = t.data + j * t.nrow;
    if (val < x[0]) return -1;
    if (val >= x[t.nrow - 1]) return t.nrow - 1;
    int lo = 0, hi = t.nrow - 1;  // x[lo] <= val < x[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (val >= x[mid]) lo = mid; else hi = mid;
    }
    return lo;
}

OCPX_HD void table_eval_all(const Table& t, int j, double val, double* out, double* slope)
{
    const int r = table_interval(t, j, val);
    const double* x = t.data + j * t.nrow;
    if (r < 0 || r >= t.nrow - 1) {
        const int e = r < 0 ? 0 : t.nrow - 1;
        for (int k = 0; k < t.ncol; k++) {
            if (slope) slope[k] = 0;
            out[k] = t.data[k * t.nrow + e];
        }
        return;
    }
    for (int k = 0; k < t.ncol; k++) {
        const double* c = t.data + k * t.nrow;
        const double s = (c[r + 1] - c[r]) / (x[r + 1] - x[r]);
        if (slope) slope[k] = s;
        out[k] = c[r] + s * (val - x[r]);
    }
}

// OCPTable::Eval (src/OCPTable.cpp:232-257): single destination column.
OCPX_HD double table_eval(const Table& t, int j, double val, int dest)
{
    const int r = table_interval(t, j, val);
    if (r < 0) return t.data[dest * t.nrow];
    if (r >= t.nrow - 1) return t.data[dest * t.nrow + t.nrow - 1];
    const double* x = t.data + j * t.nrow;
    const double* c = t.data + dest * t.nrow;
    const double k = (c[r + 1] - c[r]) / (x[r + 1] - x[r]);
    return c[r] + k * (val - x[r]);
}

// OCPTable::GetCloseRow (src/OCPTable.cpp:312-345): the nearest row, ties to
// the lower row; outside the range the end row.
OCPX_HD int table_close_row(const Table& t, int j, double val)
{
    const int r = table_interval(t, j, val);
    if (r < 0) return 0;
    if (r >= t.nrow - 1) return t.nrow - 1;
    const double* x = t.data + j * t.nrow;
    return ((val - x[r]) > (x[r + 1] - val)) ? r + 1 : r;
}

// ----------------------------------------------------------------- model --
struct Units {
    double gravity_factor;  // GRAVITY_FACTOR
    double conv_darcy;      // CONV_DARCY
    double gas_constant;    // GAS_CONSTANT
    double conv1;           // CONV1 (bbl or m3)
    double conv3;           // CONV3 (Mscf/bbl or 1)
    double conv4;           // CONV4 (degC/F -> K/R)
};

struct RockModel {
    double Pref, cp1, cp2;  // OCPRockIsoT_Linear (src/OCPRock.cpp:19-24)
};

// OCP_PVTW (src/OCPFuncPVT.cpp:22-56): Pref, Bw, Cw, mu_w, C_mu per row.
struct WaterModel {
    Table pvtw;
    double std_rho_w;
    double std_vw;
};

// SWOF + SGOF + Stone II (src/OCPFlowMethod.cpp:19-70, src/OCPFuncSAT.cpp:162-190)
struct SatModel {
    Table swof;  // Sw, krw, krow, Pcow
    Table sgof;  // Sg, krg, krog, Pcgo
    double krocw;
};

// OCPMixtureMethodK_OGW01 (src/OCPMixtureMethodK.cpp:416-759)
struct BlackOilModel {
    Table pvco;  // Pb, Rs, Bo, mu_o, Co, Cmu
    Table pvdg;  // P, Bg, mu_g
    double std_rho_o, std_rho_g, std_vo, std_vg;
};

// PR EoS + flash + LBC viscosity (src/OCPEoS.cpp, src/OCPPhaseEquilibrium.cpp,
// src/OCPMixtureMethodComp.cpp, src/OCPFuncPVT.cpp:415-576)
struct CompModel {
    int nc;                          // hydrocarbon components (NC)
    double Tc[NC_MAX], Pc[NC_MAX], Vc[NC_MAX], MW[NC_MAX];
    double OmegaA[NC_MAX], OmegaB[NC_MAX], acf[NC_MAX];
    double mwi[NC_MAX];              // PR kappa(omega), a function of acf only
    double Vshift[NC_MAX];           // Peneloux shift, already scaled
    double omb[NC_MAX * NC_MAX];     // 1 - BIC (full symmetric matrix)
    // LBC viscosity (ViscosityMethod03)
    double lbc[5];                   // coefficients, x10 as the reference stores them
    double Vcvis[NC_MAX], sqrtMW[NC_MAX], auxB[NC_MAX];
    // flash control (OCPPhaseEquilibrium::Setup, :45-64)
    int ssm_sta_maxit; double ssm_sta_tol, ssm_sta_tol2, ssm_sta_eYt, ssm_sta_Ktol, ssm_sta_dYtol;
    int nr_sta_maxit; double nr_sta_tol;
    int ssm_sp_maxit; double ssm_sp_tol2;
    int nr_sp_maxit; double nr_sp_tol;
    int rr_maxit; double rr_tol;
    int skip_psa;                    // SkipPSA on (reference default)
};

struct Model {
    int mixture;   // 0 black-oil OGW, 1 compositional
    int np, nc;    // phases (3), components incl. water
    Units units;
    RockModel rock;
    SatModel sat;
    WaterModel water;
    BlackOilModel bo;
    CompModel comp;
};

// --------------------------------------------------------------- helpers --
OCPX_HD double sq(double x) { return x * x; }
OCPX_HD double sign_d(double d) { return d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0); }
OCPX_HD bool finite_d(double x) { return (x - x) == 0.0; }

// pow(x, 1.0 / 3) for x >= 0, the cube roots of CubicRoot (src/UtilMath.cpp:15-53)
// and CalKwilson.  The exponent 1.0/3 is the double nearest 1/3, below it by
// d = 1/3 - fl(1/3) = 1.8503717077085942e-17, so
//     x^fl(1/3) = cbrt(x) * exp(-d ln x) = cbrt(x) * (1 - d ln x) + O((d ln x)^2),
// with |d ln x| < 1.4e-14 over the whole double range (the dropped term is
// below 1e-28).  The correction is at most ~62 ulp of cbrt(x), so ln x is
// needed only to single precision: ln x = e ln 2 + ln m from frexp and a
// single-precision logarithm.  Error: cbrt's (1 ulp, CUDA) plus one rounding
// of the fused multiply-add.  On GB300 this costs about a fifth of pow().
OCPX_HD double pow_third(double x)
{
#ifdef __CUDA_ARCH__
    if (!(x > 0.0) || !finite_d(x)) return pow(x, 1.0 / 3);
    const double c = cbrt(x);
    int e;
    const double m = frexp(x, &e);
    const float L = __logf((float)m) + (float)e * 0.693147180559945309f;
    const double corr = (double)L * 1.8503717077085942e-17;
    return fma(-c, corr, c);
#else
    return pow(x, 1.0 / 3);
#endif
}

}  // namespace ocpx
