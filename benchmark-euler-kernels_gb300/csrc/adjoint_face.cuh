// Transposed HLLC flux of one face: the arithmetic of the reverse step
// (adjoint.cu), in a header that also compiles as plain host C++ so that the
// CPU tests can check it against the host tangent-linear model.
//
// The flux differentiated is hllc::operator() of euler_operators/hllc.hpp:50-105.
// At exact ties (equal min/max arguments, ustar == 0 in the subsonic case)
// the derivative is the mean of the two one-sided derivatives.
#pragma once

#include <cstring>

#include "halve.cuh"

#if defined(__CUDACC__)
#define EULR_ADJ_FN __host__ __device__ __forceinline__
#else
#define EULR_ADJ_FN inline
#endif

namespace eulr {

// Reciprocal: correctly rounded on the host; on the GPU the faithful one of
// the forward step (PTX rcp.approx.ftz.f64 and one third-order Newton step,
// within one ulp), which costs three FP64 instructions.
EULR_ADJ_FN double adj_rcp(double x)
{
#if defined(__CUDA_ARCH__)
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = __fma_rn(-x, r, 1.0);
    e = __fma_rn(e, e, e);
    return __fma_rn(r, e, r);
#else
    return 1.0 / x;
#endif
}

// x * 0.5: on the GPU from the bit pattern on the integer pipe (the same bits
// as the FP64 multiply, halve.cuh), which saves an FP64 slot.
EULR_ADJ_FN double adj_half(double x)
{
#if defined(__CUDA_ARCH__)
    unsigned long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return __longlong_as_double(static_cast<long long>(halve_bits(b)));
#else
    return x * 0.5;
#endif
}

// Decisions on the integer pipe: on GB300 an FP64 compare takes a full slot
// of the FP64 pipe, which bounds the reverse step; the same decisions taken
// on the bit patterns cost nothing there.
EULR_ADJ_FN long long adj_bits(double x)
{
#if defined(__CUDA_ARCH__)
    // an opaque move: the compiler would otherwise turn some bit tests back
    // into FP64 compares, which take FP64-pipe slots
    long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
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

// Subsonic star-state branch of the upwind side q (hllc.hpp:78-102 with
// S = S_q): for the cotangent (gd, ge, gn, gt1, gt2) of the face flux it SETS
// gus (d/d ustar), gps (d/d pstar) and bq (d/d q's primitives) and returns
// d/d S_q.  a = S_q - un_q, iY = 1/(S_q - ustar).
EULR_ADJ_FN double star_branch_bar(FaceSide const& q, double a, double iY, double ustar, double pstar, double gd,
                                   double ge, double gn, double gt1, double gt2, double inv_gm1, double& gus,
                                   double& gps, FaceBar& bq)
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
    double const gE = ge * ustar;           // d/d etot_o
    double const gdo = gm * ustar;          // d/d d_o
    double const gr = gdo * q.r + gE * q.e; // d/d ratio
    double const geq = gE * r;              // d/d e (side total energy)
    double const gX = gE * iY;
    double const gY = -(gE * Xy + gr * r) * iY; // d/d (S - ustar)
    double const ga = gr * iY;                  // d/d (S - un)
    gps = gn + ge * ustar + gX * ustar;
    gus = gn * m + ge * (eo + pstar) + gm * d_o + gX * pstar - gY;
    bq.r = gdo * r + geq * q.ke;
    bq.p = geq * inv_gm1 - gX * q.un;
    bq.un = geq * (q.r * q.un) - gX * q.p - ga;
    bq.t1 = gt1 * m + geq * (q.r * q.t1);
    bq.t2 = gt2 * m + geq * (q.r * q.t2);
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
// normal and tangential momentum); with UNIT the caller has already folded
// ds into (dd, ..., dt2) and ds is not read.  SETS the cotangents of the two
// sides' primitive states, bL and bR.
//
// Written for SIMT: the upwind side q (L when ustar > 0) is selected field by
// field instead of branching on it, so a warp whose faces point both ways
// runs the star branch once, not twice; only the rare supersonic faces and
// the ustar == 0 ties take their own paths.  pstar is differentiated in its
// upwind form p_q + rc_q (ustar - un_q): the reference's mean of the two
// sides' values is the same function wherever ustar = num/den (their
// difference is (num - ustar den)/2), so the total derivative is the same.
template <bool UNIT = false>
EULR_ADJ_FN void hllc_bar(FaceSide const& L, FaceSide const& R, double dd, double de, double dn, double dt1,
                          double dt2, double ds, double inv_gm1, FaceBar& bL, FaceBar& bR)
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
    double const gd = UNIT ? dd : ds * dd;
    double const ge = UNIT ? de : ds * de;
    double const gn = UNIT ? dn : ds * dn;
    double const gt1 = UNIT ? dt1 : ds * dt1;
    double const gt2 = UNIT ? dt2 : ds * dt2;

    FaceSide q; // the upwind side's fields the branches read
    q.r = left ? L.r : R.r;
    q.p = left ? L.p : R.p;
    q.un = left ? L.un : R.un;
    q.t1 = left ? L.t1 : R.t1;
    q.t2 = left ? L.t2 : R.t2;
    q.e = left ? L.e : R.e;
    q.ke = left ? L.ke : R.ke;
    double const qrc = left ? rcL : rcR;

    FaceBar bq;
    if (adj_pos(SL) || adj_neg(SR)) {
        // S_L * S_R > 0: the flux is the upwind side's physical flux
        double const m = q.r * q.un;
        double const gm = gd + gn * q.un + gt1 * q.t1 + gt2 * q.t2;
        double const geq = ge * q.un;
        bq.un = gn * m + ge * (q.e + q.p) + gm * q.r + geq * (q.r * q.un);
        bq.r = gm * q.un + geq * q.ke;
        bq.p = gn + ge * q.un + geq * inv_gm1;
        bq.t1 = gt1 * m + geq * (q.r * q.t1);
        bq.t2 = gt2 * m + geq * (q.r * q.t2);
        bL.r = left ? bq.r : 0.0;
        bL.p = left ? bq.p : 0.0;
        bL.un = left ? bq.un : 0.0;
        bL.t1 = left ? bq.t1 : 0.0;
        bL.t2 = left ? bq.t2 : 0.0;
        bR.r = left ? 0.0 : bq.r;
        bR.p = left ? 0.0 : bq.p;
        bR.un = left ? 0.0 : bq.un;
        bR.t1 = left ? 0.0 : bq.t1;
        bR.t2 = left ? 0.0 : bq.t2;
        return;
    }

    double inv_den, ustar, gus, gps, gS;
    if (tie) {
        // ustar == 0: the mean of the two star branches, each taking half of
        // the cotangent.  With ustar = 0 the mass flux m = d_o ustar
        // vanishes, and so does every cotangent that carries a factor ustar:
        // each branch adds only its mass and energy terms to d/d ustar and
        // half of gn to d/d pstar (star_branch_bar with ustar = 0).  One
        // reciprocal gives 1/den, 1/S_L and 1/S_R.
        double const P = SL * SR;
        double const Rr = adj_rcp(den * P);
        inv_den = P * Rr;
        ustar = 0.0;
        double const pstar = q.p - qrc * q.un; // both sides' values agree at num == 0
        double const hd = adj_half(gd), he = adj_half(ge), ht1 = adj_half(gt1), ht2 = adj_half(gt2);
        gus = tie_branch_bar(L, aL, (den * SR) * Rr, pstar, hd, he, ht1, ht2) +
              tie_branch_bar(R, aR, (den * SL) * Rr, pstar, hd, he, ht1, ht2);
        gps = gn;
        gS = 0.0;
        bq.r = 0.0;
        bq.p = 0.0;
        bq.un = 0.0;
        bq.t1 = 0.0;
        bq.t2 = 0.0;
    } else {
        // One reciprocal gives 1/den and 1/(S - ustar): with Z = S den - num,
        // S - ustar = Z/den, so 1/den = Z R and 1/(S - ustar) = den^2 R for R = 1/(den Z).
        double const Z = (left ? SL : SR) * den - num;
        double const Rr = adj_rcp(den * Z);
        inv_den = Z * Rr;
        double const iY0 = (den * den) * Rr;
        ustar = num * inv_den;
        double const pstar = q.p + qrc * (ustar - q.un);
        gS = star_branch_bar(q, left ? aL : aR, iY0, ustar, pstar, gd, ge, gn, gt1, gt2, inv_gm1, gus, gps, bq);
    }

    // pstar = p_q + rc_q (ustar - un_q)
    bq.p += gps;
    bq.un -= gps * qrc;
    gus += gps * qrc;
    double const grcq = gps * (ustar - q.un);
    // to the upwind side
    bL.r = left ? bq.r : 0.0;
    bL.p = left ? bq.p : 0.0;
    bL.un = left ? bq.un : 0.0;
    bL.t1 = left ? bq.t1 : 0.0;
    bL.t2 = left ? bq.t2 : 0.0;
    bR.r = left ? 0.0 : bq.r;
    bR.p = left ? 0.0 : bq.p;
    bR.un = left ? 0.0 : bq.un;
    bR.t1 = left ? 0.0 : bq.t1;
    bR.t2 = left ? 0.0 : bq.t2;
    double grcL = left ? grcq : 0.0;
    double grcR = left ? 0.0 : grcq;
    double gSL = left ? gS : 0.0;
    double gSR = left ? 0.0 : gS;
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
    // S_L = umin - cmax, S_R = umax + cmax (equal un: half to each side)
    double const hs = adj_half(gSL + gSR);
    bL.un += u_lt ? gSL : (u_gt ? gSR : hs);
    bR.un += u_lt ? gSR : (u_gt ? gSL : hs);
    double const gc = gSR - gSL;
    double const gcL = c_lt ? 0.0 : (c_gt ? gc : adj_half(gc));
    double const gcR = gc - gcL;
    bL.p += gcL * L.cp;
    bL.r += gcL * L.cr;
    bR.p += gcR * R.cp;
    bR.r += gcR * R.cr;
}

} // namespace eulr
