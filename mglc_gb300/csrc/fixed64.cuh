// fixed64.cuh -- 64-bit fixed-point (Q55) arithmetic for the FX64 form of
// the lid-driven cavity step.
//
// GB300 executes FP64 adds and multiplies at about 1.6 per clock per SM,
// against about 50 64-bit integer adds; the IEEE FP64 step spends ~205 FP64
// instructions per cell and is bound by that unit.  The FX64 form keeps FP64
// storage but runs the collision on signed 64-bit integers holding
// value * 2^55 (range +-256, resolution 2^-55 ~ 2.8e-17):
//   * the forward and inverse moment transforms (integer coefficients) are
//     exact integer sums, where FP64 rounds every partial sum (the energy
//     moment alone reaches ~10, an FP64 ulp of 1.8e-15);
//   * products of fixed-point values (velocities, equilibrium terms) take the
//     high part of the 128-bit product (error <= 2^-55);
//   * relaxation rates and other constants below 1/2 are held as
//     round(c * 2^64) and applied with one high multiply;
//   * conversions to and from FP64 are integer bit operations: a population
//     is rounded to 2^-55 (exact when |f| >= 1/8), a result is rounded once
//     to the nearest double (ties to even).
// Range: every intermediate stays below 256 in magnitude while |f_i| < 1,
// 1/4 <= rho < 2 and |u_x|, |u_y|, |u_z| < 1/2 (a lattice flow at Mach ~0.9;
// cavity flows keep rho within a few percent of 1 and |u| near U0).  A cell
// outside that box, or holding a NaN or an infinity, writes NaN, so a
// diverged solve shows up in the residual and the totals as it does in FP64.
#pragma once
#include <cstdint>

#include "lbm_common.cuh"

namespace mglc {

constexpr int FXQ = 55;
constexpr long long FX_ONE = 1LL << FXQ;

// |x| >= 1, infinity or NaN: the exponent field is at least 1023
__device__ __forceinline__ bool fx_bad(double x) {
    return ((unsigned)(__double_as_longlong(x) >> 52) & 0x7FFu) >= 1023u;
}

// |x| >= 2, infinity or NaN (temperatures, which reach 1 at a hot wall, and
// their populations)
__device__ __forceinline__ bool fx_bad2(double x) {
    return ((unsigned)(__double_as_longlong(x) >> 52) & 0x7FFu) >= 1024u;
}

// FP64 -> Q55 for |x| < 256: exact for |x| >= 1/8, rounded to nearest
// (ties away from zero) below; larger inputs give unspecified values (the
// callers replace such cells by NaN).
// Branch-free: the 53-bit significand is placed at bit 62 and shifted right
// by 1030 - e (clamped), so one shift direction serves every exponent.
__device__ __forceinline__ long long d2q(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned hi = (unsigned)((unsigned long long)b >> 32);
    const int e = (int)((hi >> 20) & 0x7FFu);
    const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const unsigned long long v = m << 10;  // value * 2^55 = v >> (1030 - e)
    int s = (1075 - FXQ + 10) - e;         // >= 1 for |x| < 256
    s = s > 63 ? 63 : (s < 1 ? 1 : s);
    const long long r = (long long)(((v >> (s - 1)) + 1ull) >> 1);
    const long long rz = e ? r : 0LL;       // zero and subnormal inputs
    return b < 0 ? -rz : rz;
}

// Q55 -> FP64, rounded to nearest (ties to even); branch-free
__device__ __forceinline__ double q2d(long long v) {
    const long long sg = v >> 63;
    unsigned long long a = (unsigned long long)((v ^ sg) - sg);
    const int lz = __clzll((long long)a);  // 64 for a == 0
    a = lz < 64 ? a << lz : 0ull;
    unsigned long long mant = a >> 11;
    const unsigned rb = (unsigned)(a & 0x7FFu);
    mant += (rb > 0x400u || (rb == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    // value = 1.x * 2^(63 - lz - 55): biased exponent 1023 + 63 - 55 - lz; the
    // implicit bit of mant adds one to the exponent field (two when rounding
    // carried into bit 53), so the field starts one lower
    const unsigned long long bits =
        a ? ((unsigned long long)(1022 + 63 - FXQ - lz) << 52) + mant : 0ull;
    return __longlong_as_double((long long)(bits | ((unsigned long long)sg << 63)));
}

// The same two conversions on the FP64 unit, which the fixed-point collision
// otherwise leaves idle: scaling by 2^+-55 is an exact integer add on the
// exponent field, the conversion itself is one cvt instruction.
// q2d_cvt(v) == q2d(v) for every v; d2q_cvt rounds ties to even (d2q: away
// from zero), which differs only for inputs below 1/8 that end in exactly
// half a unit of 2^-55.
__device__ __forceinline__ double q2d_cvt(long long v) {
    const long long b = __double_as_longlong((double)v);  // round to nearest even
    return __longlong_as_double(v ? b - ((long long)FXQ << 52) : 0LL);
}
__device__ __forceinline__ long long d2q_cvt(double x) {
    return __double2ll_rn(__longlong_as_double(__double_as_longlong(x) + ((long long)FXQ << 52)));
}

// (a * b) >> 55 for signed Q55 values (floor of the exact product)
__device__ __forceinline__ long long qmul(long long a, long long b) {
    const long long hi = __mul64hi(a, b);
    const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
    return (long long)(((unsigned long long)hi << (64 - FXQ)) | (lo >> FXQ));
}
// a * c for a constant 0 <= c < 1/2 held as C = round(c * 2^64)
__device__ __forceinline__ long long qmulc(long long a, long long C) { return __mul64hi(a, C); }

// host: round(c * 2^64) for 0 <= c < 1/2
inline long long fx_const(double c) {
    long double v = (long double)c * 18446744073709551616.0L;
    return (long long)(v + 0.5L);
}

// relaxation coefficients c_k = s_k / |M_k|^2 as round(c_k * 2^64) and the
// lid term U0/6
struct FxCoef {
    long long c1, c2, c4, c9, c10, c11, c12, c13, c16;
    long long u0_6;
};
inline FxCoef make_fx_coef(const MrtCoef<double>& c, double u0) {
    FxCoef f;
    f.c1 = fx_const(c.c1); f.c2 = fx_const(c.c2); f.c4 = fx_const(c.c4); f.c9 = fx_const(c.c9);
    f.c10 = fx_const(c.c10); f.c11 = fx_const(c.c11); f.c12 = fx_const(c.c12);
    f.c13 = fx_const(c.c13); f.c16 = fx_const(c.c16);
    f.u0_6 = fx_const(u0 / 6.0);
    return f;
}
constexpr long long FX_THIRD = 6148914691236517205LL;  // round(2^64 / 3)

// 1 / rho for 1/4 <= rho < 2: single-precision seed from the top bits, then
// two Newton steps x <- x (2 - rho x) (seed error ~2^-22 -> 2^-44 -> 2^-55)
__device__ __forceinline__ long long fx_recip(long long rho) {
    const float rf = (float)(int)(rho >> (FXQ - 26)) * 0x1p-26f;
    long long x = (long long)__float2int_rn(__frcp_rn(rf) * 0x1p28f) << (FXQ - 28);
    x = qmul(x, 2 * FX_ONE - qmul(rho, x));
    x = qmul(x, 2 * FX_ONE - qmul(rho, x));
    return x;
}

// Lid MRT collision (collision.f90:20-189, meq(12) without rho) on Q55
// populations, in place.  FIRST: rho and u come from the stored macroscopic
// fields; otherwise from the populations (rho u = j exactly).  Returns false
// when rho or u leaves the range box.
template <bool FIRST>
__device__ __forceinline__ bool mrt_collide_fx(long long* f, long long rho_in, long long ux_in,
                                               long long uy_in, long long uz_in,
                                               const FxCoef& c, long long& rho_out) {
    using ll = long long;
    ll s1 = f[1] + f[2], d1 = f[1] - f[2];
    ll s2 = f[3] + f[4], d2 = f[3] - f[4];
    ll s3 = f[5] + f[6], d3 = f[5] - f[6];
    ll s4 = f[7] + f[10], d4 = f[7] - f[10];
    ll s5 = f[9] + f[8], d5 = f[9] - f[8];
    ll s6 = f[11] + f[14], d6 = f[11] - f[14];
    ll s7 = f[13] + f[12], d7 = f[13] - f[12];
    ll s8 = f[15] + f[18], d8 = f[15] - f[18];
    ll s9 = f[17] + f[16], d9 = f[17] - f[16];
    const ll sa = s1 + s2 + s3;
    const ll sxy = s4 + s5, sxz = s6 + s7, syz = s8 + s9;
    const ll se = sxy + sxz + syz;
    const ll ex_ = (d4 + d5) + (d6 + d7);
    const ll ey_ = (d4 - d5) + (d8 + d9);
    const ll ez_ = (d6 - d7) + (d8 - d9);
    ll rho, ux, uy, uz, rux, ruy, ruz;
    if (FIRST) {
        rho = rho_in;
        ux = ux_in;
        uy = uy_in;
        uz = uz_in;
        rux = qmul(rho, ux);
        ruy = qmul(rho, uy);
        ruz = qmul(rho, uz);
    } else {
        rho = f[0] + sa + se;
        rux = d1 + ex_;
        ruy = d2 + ey_;
        ruz = d3 + ez_;
        const ll inv = fx_recip(rho);
        ux = qmul(rux, inv);
        uy = qmul(ruy, inv);
        uz = qmul(ruz, inv);
    }
    rho_out = rho;
    const ll uh = FX_ONE / 2;
    const bool ok = rho >= FX_ONE / 4 && rho < 2 * FX_ONE && ux > -uh && ux < uh && uy > -uh &&
                    uy < uh && uz > -uh && uz < uh;
    const ll m1 = -30 * f[0] - 11 * sa + 8 * se;
    const ll m2 = 12 * f[0] - 4 * sa + se;
    const ll m4 = -4 * d1 + ex_;
    const ll m6 = -4 * d2 + ey_;
    const ll m8 = -4 * d3 + ez_;
    const ll m9 = 2 * s1 - (s2 + s3) + (sxy + sxz) - 2 * syz;
    const ll m10 = -4 * s1 + 2 * (s2 + s3) + (sxy + sxz) - 2 * syz;
    const ll m11 = (s2 - s3) + (sxy - sxz);
    const ll m12 = -2 * (s2 - s3) + (sxy - sxz);
    const ll m13 = s4 - s5;
    const ll m14 = s8 - s9;
    const ll m15 = s6 - s7;
    const ll m16 = (d4 + d5) - (d6 + d7);
    const ll m17 = (d5 - d4) + (d8 + d9);
    const ll m18 = (d6 - d7) - (d8 - d9);
    // equilibrium parts
    const ll ux2 = qmul(ux, ux), uy2 = qmul(uy, uy), uz2 = qmul(uz, uz);
    const ll rusq = qmul(rho, ux2 + uy2 + uz2);
    const ll p9 = 2 * ux2 - uy2 - uz2;
    const ll p11 = uy2 - uz2;
    const ll rp9 = qmul(rho, p9);
    const ll n1 = m1 - (-11 * rho + 19 * rusq);
    const ll n2 = m2 - (3 * rho - ((11 * rusq) >> 1));
    const ll n4 = m4 + qmulc(2 * rux, FX_THIRD);
    const ll n6 = m6 + qmulc(2 * ruy, FX_THIRD);
    const ll n8 = m8 + qmulc(2 * ruz, FX_THIRD);
    const ll n9 = m9 - rp9;
    const ll n10 = m10 + (rp9 >> 1);
    const ll n11 = m11 - qmul(rho, p11);
    const ll n12 = m12 + (p11 >> 1);
    const ll n13 = m13 - qmul(rux, uy);
    const ll n14 = m14 - qmul(ruy, uz);
    const ll n15 = m15 - qmul(rux, uz);
    // r_k = c_k n_k
    const ll r1 = qmulc(n1, c.c1), r2 = qmulc(n2, c.c2);
    const ll r4 = qmulc(n4, c.c4), r6 = qmulc(n6, c.c4), r8 = qmulc(n8, c.c4);
    const ll r9 = qmulc(n9, c.c9), r10 = qmulc(n10, c.c10), r11 = qmulc(n11, c.c11);
    const ll r12 = qmulc(n12, c.c12);
    const ll r13 = qmulc(n13, c.c13), r14 = qmulc(n14, c.c13), r15 = qmulc(n15, c.c13);
    const ll r16 = qmulc(m16, c.c16), r17 = qmulc(m17, c.c16), r18 = qmulc(m18, c.c16);
    // inverse transform M^T r by pairs (r3 = r5 = r7 = 0: conserved momentum)
    const ll bax = -11 * r1 - 4 * r2;
    const ll bed = 8 * r1 + r2;
    f[0] -= -30 * r1 + 12 * r2;
    const ll A9 = -r9 + 2 * r10, B11 = r11 - 2 * r12;
    const ll S910 = r9 + r10, S1112 = r11 + r12;
    const ll X = r4, Y = r6, Z = r8;
    ll E, O;
    E = bax + (2 * r9 - 4 * r10); O = -4 * r4;
    f[1] -= E + O; f[2] -= E - O;
    E = bax + A9 + B11; O = -4 * r6;
    f[3] -= E + O; f[4] -= E - O;
    E = bax + A9 - B11; O = -4 * r8;
    f[5] -= E + O; f[6] -= E - O;
    const ll be = bed + S910;
    E = be + S1112 + r13; O = X + Y + (r16 - r17);
    f[7] -= E + O; f[10] -= E - O;
    E = be + S1112 - r13; O = X - Y + (r16 + r17);
    f[9] -= E + O; f[8] -= E - O;
    E = be - S1112 + r15; O = X + Z + (r18 - r16);
    f[11] -= E + O; f[14] -= E - O;
    E = be - S1112 - r15; O = X - Z - (r16 + r18);
    f[13] -= E + O; f[12] -= E - O;
    const ll bz = bed - 2 * S910;
    E = bz + r14; O = Y + Z + (r17 - r18);
    f[15] -= E + O; f[18] -= E - O;
    E = bz - r14; O = Y - Z + (r17 + r18);
    f[17] -= E + O; f[16] -= E - O;
    return ok;
}


// ------------------------------------------------------------ heated cavity --
// Constants of the forced D3Q19 MRT and of the D3Q7 MRT (bouyancy3d_mpi.F90:
// 641-864, 1014-1070) for the Q55 form.  Factors below 1/2 are round(c 2^64)
// (qmulc); the others are Q55 values (qmul).
struct FxThermalCoef {
    FxCoef c;                                         // relaxation c_k (u0_6 unused)
    long long h1, h2, h3, h4, h9, h10, h11, h12, h13; // (1 - s_k/2) / |M_k|^2, qmulc
    long long gbeta;                                  // g beta, qmulc
    long long omega2;                                 // 2 Omega (Q55)
    long long t_ref;                                  // Q55
    long long para_a;                                 // Q55
    long long qd_half;                                // q_d / 2 (Q55)
    long long qnu42, qnu12, qnu4;                     // q_nu / |N_k|^2, qmulc
    long long chot, ccold;                            // (6 + paraA) / 21 * T_wall (Q55)
};
inline long long fx_q55(double x) {
    long double v = (long double)x * (long double)FX_ONE;
    return (long long)(v < 0 ? v - 0.5L : v + 0.5L);
}
inline FxThermalCoef make_fx_thermal(const MrtCoef<double>& m, double gbeta, double omega_rot,
                                     double t_ref, double para_a, double qd, double qnu,
                                     double t_hot, double t_cold) {
    FxThermalCoef t;
    t.c = make_fx_coef(m, 0.0);
    t.h1 = fx_const(m.h1); t.h2 = fx_const(m.h2); t.h3 = fx_const(m.h3); t.h4 = fx_const(m.h4);
    t.h9 = fx_const(m.h9); t.h10 = fx_const(m.h10); t.h11 = fx_const(m.h11);
    t.h12 = fx_const(m.h12); t.h13 = fx_const(m.h13);
    t.gbeta = fx_const(gbeta);
    t.omega2 = fx_q55(2.0 * omega_rot);
    t.t_ref = fx_q55(t_ref);
    t.para_a = fx_q55(para_a);
    t.qd_half = fx_q55(0.5 * qd);
    t.qnu42 = fx_const(qnu / 42.0); t.qnu12 = fx_const(qnu / 12.0); t.qnu4 = fx_const(qnu / 4.0);
    t.chot = fx_q55((6.0 + para_a) / 21.0 * t_hot);
    t.ccold = fx_q55((6.0 + para_a) / 21.0 * t_cold);
    return t;
}

// Forced MRT collision of the heated cavity on Q55 populations, in place
// (meq(12) with rho; source (1 - s/2) S in moment space).  rho, u and the force
// (fx, fy, fz) are given; rux = rho u (= j + F/2 when u came from the
// populations).  Returns false when rho or u leaves the range box.
__device__ __forceinline__ bool mrt_collide_fx_forced(long long* f, long long rho, long long ux,
                                                      long long uy, long long uz, long long rux,
                                                      long long ruy, long long ruz, long long fx,
                                                      long long fy, long long fz,
                                                      const FxThermalCoef& T) {
    using ll = long long;
    const FxCoef& c = T.c;
    ll s1 = f[1] + f[2], d1 = f[1] - f[2];
    ll s2 = f[3] + f[4], d2 = f[3] - f[4];
    ll s3 = f[5] + f[6], d3 = f[5] - f[6];
    ll s4 = f[7] + f[10], d4 = f[7] - f[10];
    ll s5 = f[9] + f[8], d5 = f[9] - f[8];
    ll s6 = f[11] + f[14], d6 = f[11] - f[14];
    ll s7 = f[13] + f[12], d7 = f[13] - f[12];
    ll s8 = f[15] + f[18], d8 = f[15] - f[18];
    ll s9 = f[17] + f[16], d9 = f[17] - f[16];
    const ll sa = s1 + s2 + s3;
    const ll sxy = s4 + s5, sxz = s6 + s7, syz = s8 + s9;
    const ll se = sxy + sxz + syz;
    const ll ex_ = (d4 + d5) + (d6 + d7);
    const ll ey_ = (d4 - d5) + (d8 + d9);
    const ll ez_ = (d6 - d7) + (d8 - d9);
    const ll uh = FX_ONE / 2;
    const bool ok = rho >= FX_ONE / 4 && rho < 2 * FX_ONE && ux > -uh && ux < uh && uy > -uh &&
                    uy < uh && uz > -uh && uz < uh;
    const ll m1 = -30 * f[0] - 11 * sa + 8 * se;
    const ll m2 = 12 * f[0] - 4 * sa + se;
    const ll m4 = -4 * d1 + ex_;
    const ll m6 = -4 * d2 + ey_;
    const ll m8 = -4 * d3 + ez_;
    const ll m9 = 2 * s1 - (s2 + s3) + (sxy + sxz) - 2 * syz;
    const ll m10 = -4 * s1 + 2 * (s2 + s3) + (sxy + sxz) - 2 * syz;
    const ll m11 = (s2 - s3) + (sxy - sxz);
    const ll m12 = -2 * (s2 - s3) + (sxy - sxz);
    const ll m13 = s4 - s5;
    const ll m14 = s8 - s9;
    const ll m15 = s6 - s7;
    const ll m16 = (d4 + d5) - (d6 + d7);
    const ll m17 = (d5 - d4) + (d8 + d9);
    const ll m18 = (d6 - d7) - (d8 - d9);
    const ll ux2 = qmul(ux, ux), uy2 = qmul(uy, uy), uz2 = qmul(uz, uz);
    const ll rusq = qmul(rho, ux2 + uy2 + uz2);
    const ll p9 = 2 * ux2 - uy2 - uz2;
    const ll p11 = uy2 - uz2;
    const ll rp9 = qmul(rho, p9);
    const ll n1 = m1 - (-11 * rho + 19 * rusq);
    const ll n2 = m2 - (3 * rho - ((11 * rusq) >> 1));
    const ll n4 = m4 + qmulc(2 * rux, FX_THIRD);
    const ll n6 = m6 + qmulc(2 * ruy, FX_THIRD);
    const ll n8 = m8 + qmulc(2 * ruz, FX_THIRD);
    const ll n9 = m9 - rp9;
    const ll n10 = m10 + (rp9 >> 1);
    const ll rp11 = qmul(rho, p11);
    const ll n11 = m11 - rp11;
    const ll n12 = m12 + (rp11 >> 1);
    const ll n13 = m13 - qmul(rux, uy);
    const ll n14 = m14 - qmul(ruy, uz);
    const ll n15 = m15 - qmul(rux, uz);
    ll r1 = qmulc(n1, c.c1), r2 = qmulc(n2, c.c2);
    ll r4 = qmulc(n4, c.c4), r6 = qmulc(n6, c.c4), r8 = qmulc(n8, c.c4);
    ll r9 = qmulc(n9, c.c9), r10 = qmulc(n10, c.c10), r11 = qmulc(n11, c.c11);
    ll r12 = qmulc(n12, c.c12);
    ll r13 = qmulc(n13, c.c13), r14 = qmulc(n14, c.c13), r15 = qmulc(n15, c.c13);
    const ll r16 = qmulc(m16, c.c16), r17 = qmulc(m17, c.c16), r18 = qmulc(m18, c.c16);
    // source terms (evolution_f.F90:107-129): r -= h S
    const ll ufx = qmul(ux, fx), vfy = qmul(uy, fy), wfz = qmul(uz, fz);
    const ll uf = ufx + vfy + wfz;
    r1 -= qmulc(38 * uf, T.h1);
    r2 += qmulc(11 * uf, T.h2);
    const ll r3 = -qmulc(fx, T.h3), r5 = -qmulc(fy, T.h3), r7 = -qmulc(fz, T.h3);
    r4 += qmulc(qmulc(2 * fx, FX_THIRD), T.h4);
    r6 += qmulc(qmulc(2 * fy, FX_THIRD), T.h4);
    r8 += qmulc(qmulc(2 * fz, FX_THIRD), T.h4);
    r9 -= qmulc(4 * ufx - 2 * vfy - 2 * wfz, T.h9);
    r10 -= qmulc(-2 * ufx + vfy + wfz, T.h10);
    r11 -= qmulc(2 * vfy - 2 * wfz, T.h11);
    r12 -= qmulc(wfz - vfy, T.h12);
    r13 -= qmulc(qmul(ux, fy) + qmul(uy, fx), T.h13);
    r14 -= qmulc(qmul(uy, fz) + qmul(uz, fy), T.h13);
    r15 -= qmulc(qmul(ux, fz) + qmul(uz, fx), T.h13);
    // inverse transform M^T r by pairs
    const ll bax = -11 * r1 - 4 * r2;
    const ll bed = 8 * r1 + r2;
    f[0] -= -30 * r1 + 12 * r2;
    const ll A9 = -r9 + 2 * r10, B11 = r11 - 2 * r12;
    const ll S910 = r9 + r10, S1112 = r11 + r12;
    const ll X = r3 + r4, Y = r5 + r6, Z = r7 + r8;
    ll E, O;
    E = bax + (2 * r9 - 4 * r10); O = r3 - 4 * r4;
    f[1] -= E + O; f[2] -= E - O;
    E = bax + A9 + B11; O = r5 - 4 * r6;
    f[3] -= E + O; f[4] -= E - O;
    E = bax + A9 - B11; O = r7 - 4 * r8;
    f[5] -= E + O; f[6] -= E - O;
    const ll be = bed + S910;
    E = be + S1112 + r13; O = X + Y + (r16 - r17);
    f[7] -= E + O; f[10] -= E - O;
    E = be + S1112 - r13; O = X - Y + (r16 + r17);
    f[9] -= E + O; f[8] -= E - O;
    E = be - S1112 + r15; O = X + Z + (r18 - r16);
    f[11] -= E + O; f[14] -= E - O;
    E = be - S1112 - r15; O = X - Z - (r16 + r18);
    f[13] -= E + O; f[12] -= E - O;
    const ll bz = bed - 2 * S910;
    E = bz + r14; O = Y + Z + (r17 - r18);
    f[15] -= E + O; f[18] -= E - O;
    E = bz - r14; O = Y - Z + (r17 + r18);
    f[17] -= E + O; f[16] -= E - O;
    return ok;
}

// D3Q7 MRT of the temperature populations (evolution_g.F90:1-57) on Q55, in
// place: n = N g, t = q (n - neq) / |N|^2, g -= N^T t.
__device__ __forceinline__ void mrt_collide_t_fx(long long* g, long long temp, long long ux,
                                                 long long uy, long long uz,
                                                 const FxThermalCoef& T) {
    using ll = long long;
    const ll n1 = g[1] - g[2], n2 = g[3] - g[4], n3 = g[5] - g[6];
    const ll sx = g[1] + g[2], sy = g[3] + g[4], sz = g[5] + g[6];
    const ll n4 = -6 * g[0] + (sx + sy + sz);
    const ll n5 = 2 * sx - (sy + sz);
    const ll n6 = sy - sz;
    const ll t1 = qmul(n1 - qmul(temp, ux), T.qd_half);
    const ll t2 = qmul(n2 - qmul(temp, uy), T.qd_half);
    const ll t3 = qmul(n3 - qmul(temp, uz), T.qd_half);
    const ll t4 = qmulc(n4 - qmul(temp, T.para_a), T.qnu42);
    const ll t5 = qmulc(n5, T.qnu12);
    const ll t6 = qmulc(n6, T.qnu4);
    g[0] -= -6 * t4;
    const ll ex5 = t4 + 2 * t5;
    const ll ey5 = t4 - t5;
    g[1] -= ex5 + t1; g[2] -= ex5 - t1;
    g[3] -= (ey5 + t6) + t2; g[4] -= (ey5 + t6) - t2;
    g[5] -= (ey5 - t6) + t3; g[6] -= (ey5 - t6) - t3;
}

}  // namespace mglc
