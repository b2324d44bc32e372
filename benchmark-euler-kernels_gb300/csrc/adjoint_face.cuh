// Transposed HLLC flux of one face: the arithmetic of the reverse step
// (adjoint.cu), in a header that also compiles as plain host C++ so that the
// CPU tests can check it against the host tangent-linear model.
//
// The flux differentiated is hllc::operator() of euler_operators/hllc.hpp:50-105.
// At exact ties (equal min/max arguments, ustar == 0 in the subsonic case)
// the derivative is the mean of the two one-sided derivatives.
#pragma once

#include <cstring>

#if defined(__CUDACC__)
#define EULR_ADJ_FN __host__ __device__ __forceinline__
#else
#define EULR_ADJ_FN inline
#endif

namespace eulr {

// Correctly rounded reciprocal (the device instruction sequence on the GPU).
EULR_ADJ_FN double adj_rcp(double x)
{
#if defined(__CUDA_ARCH__)
    return __drcp_rn(x);
#else
    return 1.0 / x;
#endif
}

// Decisions on the integer pipe: on GB300 an FP64 compare takes a full slot
// of the FP64 pipe, which bounds the reverse step; the same decisions taken
// on the bit patterns cost nothing there.
EULR_ADJ_FN long long adj_bits(double x)
{
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// Integer key with the order of the doubles, -0 and +0 equal (ties must
// see them as one value).
EULR_ADJ_FN long long adj_key(double x)
{
    long long const b = adj_bits(x);
    return (b << 1) == 0 ? 0 : (b ^ ((b >> 63) & 0x7fffffffffffffffLL));
}

EULR_ADJ_FN bool adj_neg(double x) // x < 0
{
    long long const b = adj_bits(x);
    return b < 0 && (b << 1) != 0;
}

EULR_ADJ_FN bool adj_pos(double x) // x > 0 (for non-NaN x)
{
    return adj_bits(x) > 0;
}

EULR_ADJ_FN bool adj_zero(double x) // x == +0 or -0
{
    return (adj_bits(x) << 1) == 0;
}

// One side of a face in the face frame: normal velocity un, tangential t1, t2.
struct FaceSide {
    double r, p, un, t1, t2;
    double c, cp, cr; // sound speed, dc/dp, dc/drho
    double e, ke;     // total energy per volume, kinetic energy per mass
};

struct FaceBar {
    double r, p, un, t1, t2;
};

EULR_ADJ_FN void zero(FaceBar& b) { b.r = b.p = b.un = b.t1 = b.t2 = 0.0; }

// Subsonic star-state branch of side Q (hllc.hpp:78-102 with S = S_Q, q = Q):
// adds its transposed contribution for the cotangent (gd, ge, gn, gt1, gt2)
// to gus (d/d ustar), gps (d/d pstar) and bq, and returns d/d S_Q.
EULR_ADJ_FN double star_branch_bar(FaceSide const& q, double S, double a, double iY, double ustar,
                                                  double pstar, double gd, double ge, double gn, double gt1,
                                                  double gt2, double inv_gm1, double& gus, double& gps, FaceBar& bq)
{
    // forward: ratio = (S - un)/(S - ustar), d_o = ratio rho, etot_o = ratio e + X/(S - ustar),
    // X = pstar ustar - p un; fluxes m = d_o ustar; (m, (etot_o + pstar) ustar, m ustar + pstar, m t1, m t2)
    double const r = a * iY;
    double const X = pstar * ustar - q.p * q.un;
    double const Xy = X * iY;
    double const d_o = r * q.r;
    double const eo = r * q.e + Xy;
    double const m = d_o * ustar;
    double const gm = gd + gn * ustar + gt1 * q.t1 + gt2 * q.t2;
    gus += gn * m + ge * (eo + pstar) + gm * d_o;
    gps += gn + ge * ustar;
    double const gE = ge * ustar;          // d/d etot_o
    double const gdo = gm * ustar;         // d/d d_o
    double const gr = gdo * q.r + gE * q.e; // d/d ratio
    double const geq = gE * r;             // d/d e (side total energy)
    double const gX = gE * iY;
    double const gY = -(gE * Xy + gr * r) * iY; // d/d (S - ustar)
    double const ga = gr * iY;                  // d/d (S - un)
    gps += gX * ustar;
    gus += gX * pstar - gY;
    bq.r += gdo * r + geq * q.ke;
    bq.p += geq * inv_gm1 - gX * q.un;
    bq.un += geq * (q.r * q.un) - gX * q.p - ga;
    bq.t1 += gt1 * m + geq * (q.r * q.t1);
    bq.t2 += gt2 * m + geq * (q.r * q.t2);
    return gY + ga;
}

// star_branch_bar at ustar == 0 (iS = 1/S_Q): returns the branch's d/d ustar;
// its d/d pstar is gn and it adds nothing to bq or d/d S_Q.
EULR_ADJ_FN double tie_branch_bar(FaceSide const& q, double a, double iS, double pstar, double gd, double ge,
                                  double gt1, double gt2)
{
    double const r = a * iS;
    double const d_o = r * q.r;
    double const eo = r * q.e - (q.p * q.un) * iS;
    double const gm = gd + gt1 * q.t1 + gt2 * q.t2;
    return ge * (eo + pstar) + gm * d_o;
}

// Transposed HLLC flux of one face (hllc.hpp:50-105).  The cotangent of the
// face flux is ds * (dd, de, dn, dt1, dt2) in the face frame (mass, energy,
// normal and tangential momentum; hds = ds / 2); adds the cotangents of both
// sides' primitive states to bL and bR.
EULR_ADJ_FN void hllc_bar(FaceSide const& L, FaceSide const& R, double dd, double de, double dn, double dt1,
                          double dt2, double ds, double hds, double inv_gm1, FaceBar& bL, FaceBar& bR)
{
    // S_L = min(un_L, un_R) - max(c_L, c_R), S_R = max(un_L, un_R) + max(c_L, c_R)
    long long const kuL = adj_key(L.un), kuR = adj_key(R.un);
    long long const kcL = adj_key(L.c), kcR = adj_key(R.c);
    bool const u_lt = kuL < kuR;
    bool const u_gt = kuR < kuL;
    bool const c_lt = kcL < kcR;
    bool const c_gt = kcR < kcL;
    double const umin = u_gt ? R.un : L.un;
    double const umax = u_lt ? R.un : L.un;
    double const cmax = c_lt ? R.c : L.c;
    double const SL = umin - cmax;
    double const SR = umax + cmax;
    double const aL = SL - L.un;
    double const aR = SR - R.un;
    double const rcL = L.r * aL;
    double const rcR = R.r * aR;
    double const num = (R.p - L.p) + rcL * L.un - rcR * R.un;
    double const den = rcL - rcR; // rcL <= 0 <= rcR: den < 0, so ustar > 0 exactly when num < 0
    bool const left = adj_neg(num);
    bool const tie = adj_zero(num);
    // at a tie each of the two branches takes half of the cotangent
    double const sc = tie ? hds : ds;
    double const gd = sc * dd, ge = sc * de, gn = sc * dn, gt1 = sc * dt1, gt2 = sc * dt2;

    if (adj_pos(SL) || adj_neg(SR)) {
        // S_L * S_R > 0: the flux is the upwind side's physical flux (ustar > 0 picks L)
        FaceSide const& q = left ? L : R;
        FaceBar& bq = left ? bL : bR;
        double const m = q.r * q.un;
        double const gm = gd + gn * q.un + gt1 * q.t1 + gt2 * q.t2;
        double const geq = ge * q.un;
        bq.un += gn * m + ge * (q.e + q.p) + gm * q.r + geq * (q.r * q.un);
        bq.r += gm * q.un + geq * q.ke;
        bq.p += gn + ge * q.un + geq * inv_gm1;
        bq.t1 += gt1 * m + geq * (q.r * q.t1);
        bq.t2 += gt2 * m + geq * (q.r * q.t2);
        return;
    }

    double inv_den, ustar, pstar;
    double gus = 0.0, gps = 0.0, gSL = 0.0, gSR = 0.0;
    if (tie) {
        // ustar == 0: the mean of the two star branches.  With ustar = 0 the
        // mass flux m = d_o ustar vanishes, and so does every cotangent that
        // carries a factor ustar: each branch adds only its mass and energy
        // terms to d/d ustar and gn to d/d pstar (star_branch_bar with ustar = 0).
        // One reciprocal gives 1/den, 1/S_L and 1/S_R.
        double const P = SL * SR;
        double const Rr = adj_rcp(den * P);
        inv_den = P * Rr;
        ustar = 0.0;
        pstar = 0.5 * (L.p + R.p - rcL * L.un - rcR * R.un);
        gus = tie_branch_bar(L, aL, (den * SR) * Rr, pstar, gd, ge, gt1, gt2) +
              tie_branch_bar(R, aR, (den * SL) * Rr, pstar, gd, ge, gt1, gt2);
        gps = 2.0 * gn;
    } else {
        // One reciprocal gives 1/den and 1/(S - ustar): with Z = S den - num,
        // S - ustar = Z/den, so 1/den = Z R and 1/(S - ustar) = den^2 R for R = 1/(den Z).
        double const S0 = left ? SL : SR;
        double const Z = S0 * den - num;
        double const Rr = adj_rcp(den * Z);
        inv_den = Z * Rr;
        double const iY0 = (den * den) * Rr;
        ustar = num * inv_den;
        pstar = 0.5 * (L.p + R.p + rcL * (ustar - L.un) + rcR * (ustar - R.un));
        if (left) {
            gSL = star_branch_bar(L, SL, aL, iY0, ustar, pstar, gd, ge, gn, gt1, gt2, inv_gm1, gus, gps, bL);
        } else {
            gSR = star_branch_bar(R, SR, aR, iY0, ustar, pstar, gd, ge, gn, gt1, gt2, inv_gm1, gus, gps, bR);
        }
    }

    // pstar = (p_L + p_R + rc_L (ustar - un_L) + rc_R (ustar - un_R)) / 2
    double const h = 0.5 * gps;
    bL.p += h;
    bR.p += h;
    double grcL = h * (ustar - L.un);
    double grcR = h * (ustar - R.un);
    gus += h * (rcL + rcR);
    bL.un -= h * rcL;
    bR.un -= h * rcR;
    // ustar = num / den
    double const gnum = gus * inv_den;
    double const gden = -gnum * ustar;
    bR.p += gnum;
    bL.p -= gnum;
    grcL += gnum * L.un + gden;
    grcR -= gnum * R.un + gden;
    bL.un += gnum * rcL;
    bR.un -= gnum * rcR;
    // rc = rho (S - un)
    bL.r += grcL * aL;
    bR.r += grcR * aR;
    double const gaL = grcL * L.r;
    double const gaR = grcR * R.r;
    gSL += gaL;
    gSR += gaR;
    bL.un -= gaL;
    bR.un -= gaR;
    // S_L = umin - cmax, S_R = umax + cmax
    if (u_lt) {
        bL.un += gSL;
        bR.un += gSR;
    } else if (u_gt) {
        bR.un += gSL;
        bL.un += gSR;
    } else {
        double const hs = 0.5 * (gSL + gSR);
        bL.un += hs;
        bR.un += hs;
    }
    double const gc = gSR - gSL;
    double const gcL = c_lt ? 0.0 : (c_gt ? gc : 0.5 * gc);
    double const gcR = gc - gcL;
    bL.p += gcL * L.cp;
    bL.r += gcL * L.cr;
    bR.p += gcR * R.cp;
    bR.r += gcR * R.cr;
}

} // namespace eulr
