// lbm_common.cuh -- D3Q19 / D3Q7 lattice tables and the fused MRT collision
// shared by every step kernel.
//
// Velocity ordering and weights follow the reference
// (MPI/Lid_driven_cavity/fortran/3d/mpi_3d_blocked/commondata.f90:29-40):
//   0; +-x (1,2); +-y (3,4); +-z (5,6); (+1,+1,0) (-1,+1,0) (+1,-1,0) (-1,-1,0) (7..10);
//   (+1,0,+1) (-1,0,+1) (+1,0,-1) (-1,0,-1) (11..14); (0,+1,+1) (0,-1,+1) (0,+1,-1) (0,-1,-1) (15..18).
// The moment basis is the reference's M (collision.f90:20-70).  Two
// algebraically equal evaluations of the collision are kept:
//  - the moment form (mrt_collide, mrt_collide_t)
//        f_post = f - M^-1 r,   r_k = s_k (m_k - meq_k) - (1 - s_k/2) S_k,
//    with M^-1 = M^T diag(1/|M_k|^2) and opposite-direction pairs sharing
//    their even/odd parts, about half the operations of the literal
//    m -> m_post -> M^-1 m_post;
//  - the pair form (trt_collide_lid, trt_collide_forced, trt_collide_t): the
//    reference relaxes all even non-conserved moments at one rate and all odd
//    ones at another, so the collision is a two-relaxation-time update of
//    each opposite pair, about 3/4 of the moment form's operations.
// Results differ from the literal form only by rounding (a few ulp per step).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mglc {

constexpr int Q19 = 19;
constexpr int Q7 = 7;
__host__ __device__ constexpr int ex19(int a) {
    return (a == 1 || a == 7 || a == 9 || a == 11 || a == 13) ? 1
         : (a == 2 || a == 8 || a == 10 || a == 12 || a == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ey19(int a) {
    return (a == 3 || a == 7 || a == 8 || a == 15 || a == 17) ? 1
         : (a == 4 || a == 9 || a == 10 || a == 16 || a == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez19(int a) {
    return (a == 5 || a == 11 || a == 12 || a == 15 || a == 16) ? 1
         : (a == 6 || a == 13 || a == 14 || a == 17 || a == 18) ? -1 : 0;
}
// opposite direction
__host__ __device__ constexpr int opp19(int a) {
    return a == 0 ? 0 : (a <= 6 ? (a % 2 ? a + 1 : a - 1)
         : (a == 7 ? 10 : a == 10 ? 7 : a == 8 ? 9 : a == 9 ? 8
         : a == 11 ? 14 : a == 14 ? 11 : a == 12 ? 13 : a == 13 ? 12
         : a == 15 ? 18 : a == 18 ? 15 : a == 16 ? 17 : 16));
}
__host__ __device__ constexpr double w19(int a) {
    return a == 0 ? 1.0 / 3.0 : (a <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// Relaxation coefficients folded with 1/|M_k|^2 (host-computed in FP64).
// c_k = s_k / |M_k|^2, h_k = (1 - s_k/2) / |M_k|^2.
// snu, le = snu/2, lo = sq/2: the two rates of the pair form;
// ke2 = (1 - le)/le and ko = (1 - lo)/(2 lo): its force terms.
template <typename T>
struct MrtCoef {
    T c1, c2, c4, c9, c10, c11, c12, c13, c16;
    T h1, h2, h3, h4, h9, h10, h11, h12, h13;
    T snu, le, lo, ke2, ko;
};

inline MrtCoef<double> make_mrt_coef(double snu, double sq) {
    MrtCoef<double> c;
    c.snu = snu; c.le = 0.5 * snu; c.lo = 0.5 * sq;
    c.ke2 = (1.0 - c.le) / c.le; c.ko = (1.0 - c.lo) / (2.0 * c.lo);
    c.c1 = snu / 2394.0; c.c2 = snu / 252.0; c.c4 = sq / 40.0;
    c.c9 = snu / 36.0; c.c10 = snu / 72.0; c.c11 = snu / 12.0; c.c12 = snu / 24.0;
    c.c13 = snu / 4.0; c.c16 = sq / 8.0;
    c.h1 = (1.0 - 0.5 * snu) / 2394.0; c.h2 = (1.0 - 0.5 * snu) / 252.0; c.h3 = 1.0 / 10.0;
    c.h4 = (1.0 - 0.5 * sq) / 40.0; c.h9 = (1.0 - 0.5 * snu) / 36.0;
    c.h10 = (1.0 - 0.5 * snu) / 72.0; c.h11 = (1.0 - 0.5 * snu) / 12.0;
    c.h12 = (1.0 - 0.5 * snu) / 24.0; c.h13 = (1.0 - 0.5 * snu) / 4.0;
    return c;
}
template <typename T>
inline MrtCoef<T> cast_coef(const MrtCoef<double>& d) {
    MrtCoef<T> c;
    c.c1 = (T)d.c1; c.c2 = (T)d.c2; c.c4 = (T)d.c4; c.c9 = (T)d.c9; c.c10 = (T)d.c10;
    c.c11 = (T)d.c11; c.c12 = (T)d.c12; c.c13 = (T)d.c13; c.c16 = (T)d.c16;
    c.h1 = (T)d.h1; c.h2 = (T)d.h2; c.h3 = (T)d.h3; c.h4 = (T)d.h4; c.h9 = (T)d.h9;
    c.h10 = (T)d.h10; c.h11 = (T)d.h11; c.h12 = (T)d.h12; c.h13 = (T)d.h13;
    c.snu = (T)d.snu; c.le = (T)d.le; c.lo = (T)d.lo; c.ke2 = (T)d.ke2; c.ko = (T)d.ko;
    return c;
}

// Density and momentum sums of the stored populations.  For absolute storage
// this is the reference macro (sum f, sum f e); for deviation storage it is
// (rho - rho0, j).
template <typename T>
__device__ __forceinline__ void moments0(const T* f, T& rho_m, T& jx, T& jy, T& jz) {
    // pair sums keep the operation count low; order differs from the
    // reference's sequential sum only by rounding
    T s1 = f[1] + f[2], s2 = f[3] + f[4], s3 = f[5] + f[6];
    T s4 = f[7] + f[10], s5 = f[9] + f[8], s6 = f[11] + f[14], s7 = f[13] + f[12];
    T s8 = f[15] + f[18], s9 = f[17] + f[16];
    rho_m = ((f[0] + s1) + (s2 + s3)) + ((s4 + s5) + (s6 + s7)) + (s8 + s9);
    T d4 = f[7] - f[10], d5 = f[9] - f[8], d6 = f[11] - f[14], d7 = f[13] - f[12];
    T d8 = f[15] - f[18], d9 = f[17] - f[16];
    jx = (f[1] - f[2]) + (d4 + d5) + (d6 + d7);
    jy = (f[3] - f[4]) + (d4 - d5) + (d8 + d9);
    jz = (f[5] - f[6]) + (d6 - d7) + (d8 - d9);
}

// Fused MRT collision in place on f[19].
//  rho_m : sum of stored f (rho for absolute storage, rho - rho0 for deviations)
//  rho   : full density used in the equilibrium
//  (ux,uy,uz): velocity used in the equilibrium (and source)
//  FORCED: add the reference's moment-space source (evolution_f.F90:107-129)
//  LID_MEQ12: lid operator quirk, meq(12) without the factor rho (collision.f90:85)
//  msc  : scale of f, rho_m, rho and the forces (the lid quirk's meq(12), which
//         carries no rho, is multiplied by it); 1 for unscaled arithmetic
template <typename T, bool FORCED, bool LID_MEQ12>
__device__ __forceinline__ void mrt_collide(T* f, T rho_m, T rho, T ux, T uy, T uz, T fx, T fy,
                                            T fz, const MrtCoef<T>& c, T msc = T(1)) {
    const T two = T(2), four = T(4), half = T(0.5);
    // opposite pairs: (a,b) = (1,2) (3,4) (5,6) (7,10) (9,8) (11,14) (13,12) (15,18) (17,16)
    T s1 = f[1] + f[2], d1 = f[1] - f[2];
    T s2 = f[3] + f[4], d2 = f[3] - f[4];
    T s3 = f[5] + f[6], d3 = f[5] - f[6];
    T s4 = f[7] + f[10], d4 = f[7] - f[10];
    T s5 = f[9] + f[8], d5 = f[9] - f[8];
    T s6 = f[11] + f[14], d6 = f[11] - f[14];
    T s7 = f[13] + f[12], d7 = f[13] - f[12];
    T s8 = f[15] + f[18], d8 = f[15] - f[18];
    T s9 = f[17] + f[16], d9 = f[17] - f[16];
    T sa = s1 + s2 + s3;                    // axis sum
    T se = (s4 + s5) + (s6 + s7) + (s8 + s9); // edge sum
    T m1 = T(-30) * f[0] + (T(-11) * sa + T(8) * se);
    T m2 = T(12) * f[0] + (T(-4) * sa + se);
    T ex_ = (d4 + d5) + (d6 + d7);
    T ey_ = (d4 - d5) + (d8 + d9);
    T ez_ = (d6 - d7) + (d8 - d9);
    T m4 = T(-4) * d1 + ex_;
    T m6 = T(-4) * d2 + ey_;
    T m8 = T(-4) * d3 + ez_;
    T sxy = s4 + s5, sxz = s6 + s7, syz = s8 + s9;
    T m9 = two * s1 - (s2 + s3) + (sxy + sxz) - two * syz;
    T m10 = -four * s1 + two * (s2 + s3) + (sxy + sxz) - two * syz;
    T m11 = (s2 - s3) + (sxy - sxz);
    T m12 = -two * (s2 - s3) + (sxy - sxz);
    T m13 = s4 - s5;
    T m14 = s8 - s9;
    T m15 = s6 - s7;
    T m16 = (d4 + d5) - (d6 + d7);
    T m17 = (d5 - d4) + (d8 + d9);
    T m18 = (d6 - d7) - (d8 - d9);

    // equilibrium parts
    T ux2 = ux * ux, uy2 = uy * uy, uz2 = uz * uz;
    T usq = ux2 + uy2 + uz2;
    T rux = rho * ux, ruy = rho * uy, ruz = rho * uz;
    T p9 = two * ux2 - uy2 - uz2;
    T p11 = uy2 - uz2;
    T n1 = m1 - (T(-11) * rho_m + T(19) * rho * usq);
    T n2 = m2 - (T(3) * rho_m - T(5.5) * rho * usq);
    T n4 = m4 + T(2.0 / 3.0) * rux;
    T n6 = m6 + T(2.0 / 3.0) * ruy;
    T n8 = m8 + T(2.0 / 3.0) * ruz;
    T n9 = m9 - rho * p9;
    T n10 = m10 + half * (rho * p9);
    T n11 = m11 - rho * p11;
    T n12 = LID_MEQ12 ? (m12 + half * (msc * p11)) : (m12 + half * (rho * p11));
    T n13 = m13 - rux * uy;
    T n14 = m14 - ruy * uz;
    T n15 = m15 - rux * uz;

    // r~_k = c_k n_k - h_k S_k
    T r1 = c.c1 * n1, r2 = c.c2 * n2, r4 = c.c4 * n4, r6 = c.c4 * n6, r8 = c.c4 * n8;
    T r9 = c.c9 * n9, r10 = c.c10 * n10, r11 = c.c11 * n11, r12 = c.c12 * n12;
    T r13 = c.c13 * n13, r14 = c.c13 * n14, r15 = c.c13 * n15;
    T r16 = c.c16 * m16, r17 = c.c16 * m17, r18 = c.c16 * m18;
    T r3 = T(0), r5 = T(0), r7 = T(0);
    if (FORCED) {
        T uf = ux * fx + uy * fy + uz * fz;
        T ufx = ux * fx, vfy = uy * fy, wfz = uz * fz;
        r1 -= c.h1 * (T(38) * uf);
        r2 -= c.h2 * (T(-11) * uf);
        r3 = -c.h3 * fx;
        r5 = -c.h3 * fy;
        r7 = -c.h3 * fz;
        r4 -= c.h4 * (T(-2.0 / 3.0) * fx);
        r6 -= c.h4 * (T(-2.0 / 3.0) * fy);
        r8 -= c.h4 * (T(-2.0 / 3.0) * fz);
        r9 -= c.h9 * (four * ufx - two * vfy - two * wfz);
        r10 -= c.h10 * (-two * ufx + vfy + wfz);
        r11 -= c.h11 * (two * vfy - two * wfz);
        r12 -= c.h12 * (wfz - vfy);
        r13 -= c.h13 * (ux * fy + uy * fx);
        r14 -= c.h13 * (uy * fz + uz * fy);
        r15 -= c.h13 * (ux * fz + uz * fx);
    }
    // inverse transform M^T r~ by pairs
    T bax = T(-11) * r1 - four * r2;  // axis base
    T bed = T(8) * r1 + r2;           // edge base
    f[0] -= T(-30) * r1 + T(12) * r2;
    T A9 = -r9 + two * r10, B11 = r11 - two * r12;
    T S910 = r9 + r10, S1112 = r11 + r12;
    T X = r3 + r4, Y = r5 + r6, Z = r7 + r8;
    T E, O;
    // P1 (1,2)
    E = bax + (two * r9 - four * r10); O = r3 - four * r4;
    f[1] -= E + O; f[2] -= E - O;
    // P2 (3,4)
    E = bax + A9 + B11; O = r5 - four * r6;
    f[3] -= E + O; f[4] -= E - O;
    // P3 (5,6)
    E = bax + A9 - B11; O = r7 - four * r8;
    f[5] -= E + O; f[6] -= E - O;
    T be = bed + S910;
    // P4 (7,10)
    E = be + S1112 + r13; O = X + Y + (r16 - r17);
    f[7] -= E + O; f[10] -= E - O;
    // P5 (9,8)
    E = be + S1112 - r13; O = X - Y + (r16 + r17);
    f[9] -= E + O; f[8] -= E - O;
    // P6 (11,14)
    E = be - S1112 + r15; O = X + Z + (r18 - r16);
    f[11] -= E + O; f[14] -= E - O;
    // P7 (13,12)
    E = be - S1112 - r15; O = X - Z - (r16 + r18);
    f[13] -= E + O; f[12] -= E - O;
    T bz = bed - two * S910;
    // P8 (15,18)
    E = bz + r14; O = Y + Z + (r17 - r18);
    f[15] -= E + O; f[18] -= E - O;
    // P9 (17,16)
    E = bz - r14; O = Y - Z + (r17 + r18);
    f[17] -= E + O; f[16] -= E - O;
}

// The lid-driven cavity's MRT collision (collision.f90:15-202) in its pair
// form.  The reference relaxes every even non-conserved moment (e, epsilon,
// p_ww, pi_ww, p_xx-type, pi-type, p_xy, p_yz, p_xz) at Snu and every odd one
// (q_x,y,z, m_x,y,z) at Sq (collision.f90:94-112), and its basis is orthogonal,
// so M^-1 S (m - meq) = Snu [(f - feq)^+ - P_rho] + Sq [(f - feq)^- - P_j]:
// the parts of f - feq that are even and odd under e -> -e, less their
// projections on the conserved moments (s = 0 there), with feq = M^-1 meq.
// That feq is the second-order polynomial equilibrium
//     feq_i = w_i rho (1 + 3 e.u + 9/2 (e.u)^2 - 3/2 u.u)
// plus M_12^T (meq12_lid - meq12) / |M_12|^2 for the lid quirk (meq(12)
// without rho, collision.f90:85).  When rho and u come from the same
// populations (every step but the first after initial or load) the
// projections, P_rho = (sum f - rho)/19 and P_j = e.(j - rho u)/10, are at
// rounding level and are left out; CONS adds them (dr = sum f - rho,
// dj = j - rho u, in storage units) for the step that takes rho and u from
// the macro arrays.  Per opposite pair (a, b = opp a), with t = f_a + f_b,
// d = f_a - f_b, E = feq_a + feq_b (+ 2 P_rho) and O = feq_a - feq_b (+ 2 P_j):
//     f_a' = f_a - Snu/2 (t - E) - Sq/2 (d - O)
//     f_b' = f_b - Snu/2 (t - E) + Sq/2 (d - O)
// About 150 operations per cell against the moment form's 215 (FP64, ncu);
// results differ from the moment form by rounding (a few ulp).
// Arguments as mrt_collide's (rho_m: the equilibrium's density less rho0,
// rhos: its density, both in units of the storage scale; msc: the scale).
template <typename T, bool CONS = false>
__device__ __forceinline__ void trt_collide_lid(T* f, T rho_m, T rhos, T ux, T uy, T uz,
                                                const MrtCoef<T>& c, T msc = T(1),
                                                T dr = T(0), T djx = T(0), T djy = T(0),
                                                T djz = T(0)) {
    const T ux2 = ux * ux, uy2 = uy * uy, uz2 = uz * uz;
    const T usq = ux2 + uy2 + uz2;
    // feq_i = w_i (base + rhos (3 e.u + 9/2 (e.u)^2)), base = rho_m - 3/2 rhos u.u
    const T base = rho_m + T(-1.5) * rhos * usq;
    T ea = base * T(1.0 / 9.0);    // 2 w base, axis pairs (w = 1/18)
    T ee = base * T(1.0 / 18.0);   // edge pairs (w = 1/36)
    T e0 = base * T(1.0 / 3.0);    // feq_0
    const T ka = rhos * T(0.5), ke = rhos * T(0.25);            // 9 w rhos
    const T oa = rhos * T(1.0 / 3.0), oe = rhos * T(1.0 / 6.0);  // 6 w rhos
    T gx = T(0), gy = T(0), gz = T(0);  // 2 P_j per unit of e (CONS)
    if constexpr (CONS) {
        const T d19 = dr * T(2.0 / 19.0);
        ea = ea + d19;
        ee = ee + d19;
        e0 = e0 + T(0.5) * d19;
        gx = djx * T(0.2);
        gy = djy * T(0.2);
        gz = djz * T(0.2);
    }
    // lid quirk: E gains 2 M_12,a D / 24, D = (rhos - msc)(uy^2 - uz^2) / 2;
    // M_12 = -2 (y axis), +2 (z axis), +1 (xy edges), -1 (xz edges), 0 (yz)
    const T q6 = (uy2 - uz2) * ((rhos - msc) * T(1.0 / 12.0));  // D / 6
    const T q12 = q6 * T(0.5);                                    // D / 12
    const T exy = ee + q12, exz = ee - q12;
    const T le = c.le, lo = c.lo;
    auto pair = [&](int a, int b, T E, T O) {
        const T ne = (f[a] + f[b]) - E;
        const T no = (f[a] - f[b]) - O;
        const T fa = f[a] - lo * no - le * ne;
        const T fb = f[b] + lo * no - le * ne;
        f[a] = fa;
        f[b] = fb;
    };
    f[0] = f[0] - c.snu * (f[0] - e0);
    T v;
    if constexpr (CONS) {
        pair(1, 2, ea + ka * ux2, oa * ux + gx);
        pair(3, 4, (ea + ka * uy2) - q6, oa * uy + gy);
        pair(5, 6, (ea + ka * uz2) + q6, oa * uz + gz);
        v = ux + uy; pair(7, 10, exy + ke * v * v, oe * v + (gx + gy));
        v = ux - uy; pair(9, 8, exy + ke * v * v, oe * v + (gx - gy));
        v = ux + uz; pair(11, 14, exz + ke * v * v, oe * v + (gx + gz));
        v = ux - uz; pair(13, 12, exz + ke * v * v, oe * v + (gx - gz));
        v = uy + uz; pair(15, 18, ee + ke * v * v, oe * v + (gy + gz));
        v = uy - uz; pair(17, 16, ee + ke * v * v, oe * v + (gy - gz));
    } else {
        pair(1, 2, ea + ka * ux2, oa * ux);
        pair(3, 4, (ea + ka * uy2) - q6, oa * uy);
        pair(5, 6, (ea + ka * uz2) + q6, oa * uz);
        v = ux + uy; pair(7, 10, exy + ke * v * v, oe * v);
        v = ux - uy; pair(9, 8, exy + ke * v * v, oe * v);
        v = ux + uz; pair(11, 14, exz + ke * v * v, oe * v);
        v = ux - uz; pair(13, 12, exz + ke * v * v, oe * v);
        v = uy + uz; pair(15, 18, ee + ke * v * v, oe * v);
        v = uy - uz; pair(17, 16, ee + ke * v * v, oe * v);
    }
}

// The heated cavity's forced MRT collision (bouyancy3d_mpi.F90:641-864) in
// the same pair form.  Its rates are the lid operator's (even Snu, odd Sq,
// :723-741), its equilibrium has no quirk, and its moment source is M F with
// F_i = w_i (3 e.F + 9 (e.u)(e.F) - 3 u.F) (fSource, :747-765), relaxed by
// 1 - s/2 and added in full to the conserved momentum.  The velocity of the
// equilibrium is u = (j + Fp/2)/rho with the force Fp carried from the
// previous step (:998-1002), so j - rho u = -Fp/2 is not zero;
// working the three moment groups through gives, per pair,
//     f_a' = f_a - Snu/2 (t - E) - Sq/2 (d - O),  f_b' likewise with +Sq/2,
//     E = 2w (rho_m - 3/2 u.V) + 9w (e.u)(e.V),   V = rho u + (1 - le)/le F
//     O = 6w e.W + e.(F - Fp)/10,                 W = rho u + (1 - lo)/(2 lo) F
// (the equilibrium shifted by the relaxed source; the last term is what the
// unrelaxed momentum source and the carried force leave in the odd part),
// and f_0' = f_0 - Snu (f_0 - (rho_m - 3/2 u.V)/3).  About 130 operations
// against the moment form's 230; the difference is rounding.  In general the
// odd term is e.(2 (j - rho u) + F)/10, which the caller passes as dF; for
// the first step after initial or load (rho, u from the macro arrays) CONS
// also takes the density projection back out (dr = sum f - rho, as in
// trt_collide_lid).
// f, rho_m, rhos and the forces (F this step's, dF = F - Fp) in units of the
// storage scale, u unscaled; ROT: F_x, F_y (rotation) are not zero.
template <typename T, bool ROT, bool CONS = false>
__device__ __forceinline__ void trt_collide_forced(T* f, T rho_m, T rhos, T ux, T uy, T uz, T fx,
                                                   T fy, T fz, T dfx, T dfy, T dfz,
                                                   const MrtCoef<T>& c, T dr = T(0)) {
    const T rux = rhos * ux, ruy = rhos * uy, ruz = rhos * uz;
    T vx = rux, vy = ruy, wx = rux, wy = ruy;
    if (ROT) {
        vx = rux + c.ke2 * fx;
        vy = ruy + c.ke2 * fy;
        wx = rux + c.ko * fx;
        wy = ruy + c.ko * fy;
    }
    const T vz = ruz + c.ke2 * fz, wz = ruz + c.ko * fz;
    const T base = rho_m + T(-1.5) * (ux * vx + uy * vy + uz * vz);
    const T r3 = T(1.0 / 3.0), r6 = T(1.0 / 6.0), r10 = T(0.1);
    T ea = base * T(1.0 / 9.0), ee = base * T(1.0 / 18.0), e0 = base * r3;
    if constexpr (CONS) {
        const T d19 = dr * T(2.0 / 19.0);
        ea = ea + d19;
        ee = ee + d19;
        e0 = e0 + T(0.5) * d19;
    }
    // odd parts: O = e.Ga on axis pairs, e.Ge on edge pairs
    T gax = wx * r3, gay = wy * r3, gex = wx * r6, gey = wy * r6;
    if (ROT || CONS) {  // dF_x, dF_y: rotation, or j - rho u of the first step
        gax = gax + dfx * r10;
        gay = gay + dfy * r10;
        gex = gex + dfx * r10;
        gey = gey + dfy * r10;
    }
    const T gaz = wz * r3 + dfz * r10, gez = wz * r6 + dfz * r10;
    const T le = c.le, lo = c.lo;
    auto pair = [&](int a, int b, T E, T O) {
        const T ne = (f[a] + f[b]) - E;
        const T no = (f[a] - f[b]) - O;
        const T fa = f[a] - lo * no - le * ne;
        const T fb = f[b] + lo * no - le * ne;
        f[a] = fa;
        f[b] = fb;
    };
    f[0] = f[0] - c.snu * (f[0] - e0);
    pair(1, 2, ea + T(0.5) * ux * vx, gax);
    pair(3, 4, ea + T(0.5) * uy * vy, gay);
    pair(5, 6, ea + T(0.5) * uz * vz, gaz);
    const T q = T(0.25);
    pair(7, 10, ee + q * (ux + uy) * (vx + vy), gex + gey);
    pair(9, 8, ee + q * (ux - uy) * (vx - vy), gex - gey);
    pair(11, 14, ee + q * (ux + uz) * (vx + vz), gex + gez);
    pair(13, 12, ee + q * (ux - uz) * (vx - vz), gex - gez);
    pair(15, 18, ee + q * (uy + uz) * (vy + vz), gey + gez);
    pair(17, 16, ee + q * (uy - uz) * (vy - vz), gey - gez);
}

// D3Q7 MRT for the temperature populations (evolution_g.F90:1-57), in place.
// n = N g; n_post = n - q (n - neq); g_post = N^-1 n_post, with N^-1 = N^T diag(1/|N_k|^2).
// |N_k|^2 = 7, 2, 2, 2, 42, 12, 4.
template <typename T>
__device__ __forceinline__ void mrt_collide_t(T* g, T temp, T ux, T uy, T uz, T para_a, T qd,
                                              T qnu) {
    T n1 = g[1] - g[2], n2 = g[3] - g[4], n3 = g[5] - g[6];
    T sx = g[1] + g[2], sy = g[3] + g[4], sz = g[5] + g[6];
    T n4 = T(-6) * g[0] + (sx + sy + sz);
    T n5 = T(2) * sx - (sy + sz);
    T n6 = sy - sz;
    T t1 = T(0.5) * qd * (n1 - temp * ux);
    T t2 = T(0.5) * qd * (n2 - temp * uy);
    T t3 = T(0.5) * qd * (n3 - temp * uz);
    T t4 = qnu * (n4 - temp * para_a) * T(1.0 / 42.0);
    T t5 = qnu * n5 * T(1.0 / 12.0);
    T t6 = qnu * n6 * T(0.25);
    // g_post_a = g_a - sum_k N_ka t_k
    g[0] -= T(-6) * t4;
    T ex5 = t4 + T(2) * t5;
    T ey5 = t4 - t5;
    g[1] -= ex5 + t1; g[2] -= ex5 - t1;
    g[3] -= (ey5 + t6) + t2; g[4] -= (ey5 + t6) - t2;
    g[5] -= (ey5 - t6) + t3; g[6] -= (ey5 - t6) - t3;
}

// The same D3Q7 collision in pair form.  Its even non-conserved moments
// (n4..n6) relax at qnu and its odd ones (the fluxes n1..n3) at qd
// (evolution_g.F90:1-57), so g' = g - qnu (g - geq)^+ - qd (g - geq)^- with
// geq = N^-1 neq: geq_0 = T (1 - a)/7 and, per axis pair,
// E = geq_a + geq_b = T (6 + a)/21, O = geq_a - geq_b = T u_a.  The
// temperature's projection (sum g - T)/7 is at rounding level when T is the
// sum of g; CONS adds it back (dT = sum g - T) for the first step after
// initial or load, where T comes from the macro array.  About half the
// operations of the moment form.
template <typename T, bool CONS = false>
__device__ __forceinline__ void trt_collide_t(T* g, T temp, T ux, T uy, T uz, T para_a, T qd,
                                              T qnu, T dT = T(0)) {
    T e0 = temp * ((T(1) - para_a) * T(1.0 / 7.0));
    T E = temp * ((T(6) + para_a) * T(1.0 / 21.0));
    if constexpr (CONS) {
        e0 = e0 + dT * T(1.0 / 7.0);
        E = E + dT * T(2.0 / 7.0);
    }
    const T hn = T(0.5) * qnu, hd = T(0.5) * qd;
    g[0] = g[0] - qnu * (g[0] - e0);
    auto pair = [&](int a, int b, T O) {
        const T ne = (g[a] + g[b]) - E;
        const T no = (g[a] - g[b]) - O;
        const T ga = g[a] - hd * no - hn * ne;
        const T gb = g[b] + hd * no - hn * ne;
        g[a] = ga;
        g[b] = gb;
    };
    pair(1, 2, temp * ux);
    pair(3, 4, temp * uy);
    pair(5, 6, temp * uz);
}

}  // namespace mglc
