// FP64 restatement of the reference's 4-body amplitude pieces, used by the oracle only (test
// infrastructure; the engine never includes this file).
//
//   get4Vecs / getmass / Mass   src/PDFs/physics/DalitzPlotHelpers.cu:60-232
//   spin-factor helpers         include/goofit/PDFs/physics/detail/SpinHelper.h (gpuLVec, ZTspin1,
//                               ZTspin2, SpinSumV, SpinSumT, LeviCivita)
//   spin factors                src/PDFs/physics/SpinFactors.cu:83-568 (ZEMACH forms)
//   line shapes BW / SBW        src/PDFs/physics/lineshapes/BW.cu:14-121, form factors Common.cu:8-51
//   Dim5 (4-vectors -> 5 vars)  include/goofit/PDFs/physics/detail/Dim5.h:19-111, with the Vector4R
//                               conventions of MCBooster/EvtGen: `*` is the Minkowski product,
//                               dot/cross/d3mag act on the 3-vector parts
#pragma once

#include <cmath>
#include <complex>

namespace amp4 {

// 4-vector (x, y, z, E), metric (+, -, -, -) in Dot
struct LV {
    double x = 0, y = 0, z = 0, e = 0;
    LV() = default;
    LV(double X, double Y, double Z, double E) : x(X), y(Y), z(Z), e(E) {}
    double dot(const LV &o) const { return e * o.e - x * o.x - y * o.y - z * o.z; }
    double mag2() const { return dot(*this); }
    double m() const { return std::sqrt(mag2()); }
};
inline LV operator+(LV a, const LV &b) { return LV(a.x + b.x, a.y + b.y, a.z + b.z, a.e + b.e); }
inline LV operator-(LV a, const LV &b) { return LV(a.x - b.x, a.y - b.y, a.z - b.z, a.e - b.e); }
inline LV operator*(LV a, double s) { return LV(a.x * s, a.y * s, a.z * s, a.e * s); }
inline LV operator*(double s, LV a) { return LV(a.x * s, a.y * s, a.z * s, a.e * s); }

// ZTspin1: q - (q.p) p / mR^2
inline LV zt1(const LV &q, const LV &p, double mR) { return q - q.dot(p) * p * (1. / (mR * mR)); }
// SpinSumV(p, mR).Dot(v) = -v + p (p.v) / mR^2
inline LV spinSumV(const LV &p, double mR, const LV &v) { return -1.0 * v + p * (p.dot(v) / (mR * mR)); }
inline double spinSumVSandwich(const LV &p, double mR, const LV &l, const LV &r) { return l.dot(spinSumV(p, mR, r)); }
inline double spinSumTSandwich(const LV &p, double mR, const LV &lm, const LV &ln, const LV &ra, const LV &rb) {
    double manb = spinSumVSandwich(p, mR, lm, ra) * spinSumVSandwich(p, mR, ln, rb);
    double mbna = spinSumVSandwich(p, mR, lm, rb) * spinSumVSandwich(p, mR, ln, ra);
    double mnab = spinSumVSandwich(p, mR, lm, ln) * spinSumVSandwich(p, mR, ra, rb);
    return (1. / 2.) * (manb + mbna) - (1. / 3.) * mnab;
}

// Symmetric rank-2 tensor as rows X, Y, Z, E (each a 4-vector); ZTspin2 and its contraction with a vector
struct T2 {
    LV r[4]; // X, Y, Z, E rows
};
inline T2 outer(const LV &p) {
    T2 t;
    const double c[4] = {p.x, p.y, p.z, p.e};
    for(int i = 0; i < 4; ++i)
        t.r[i] = LV(c[i] * p.x, c[i] * p.y, c[i] * p.z, c[i] * p.e);
    return t;
}
inline T2 zt2(const LV &q, const LV &p, double mR) {
    LV t = zt1(q, p, mR);
    T2 tt = outer(t), uu = outer(p);
    for(auto &row : uu.r)
        row = row * (1. / (mR * mR));
    T2 g;
    g.r[0] = LV(-1, 0, 0, 0);
    g.r[1] = LV(0, -1, 0, 0);
    g.r[2] = LV(0, 0, -1, 0);
    g.r[3] = LV(0, 0, 0, 1);
    const double f = (1. / 3.) * t.mag2();
    T2 out;
    for(int i = 0; i < 4; ++i)
        out.r[i] = tt.r[i] - f * (g.r[i] - uu.r[i]);
    return out;
}
// SymmLorentzMatrix::Contract(vec) = vec.E * E - vec.X * X - vec.Y * Y - vec.Z * Z
inline LV contract(const T2 &t, const LV &v) { return v.e * t.r[3] - v.x * t.r[0] - v.y * t.r[1] - v.z * t.r[2]; }

inline double leviCivita4(const LV &p1, const LV &p2, const LV &p3, const LV &p4) {
    // the fully antisymmetric contraction eps(p1, p2, p3, p4) in the sign convention of SpinHelper.h
    const double a[4] = {p1.x, p1.y, p1.z, p1.e}, b[4] = {p2.x, p2.y, p2.z, p2.e}, c[4] = {p3.x, p3.y, p3.z, p3.e},
                 d[4] = {p4.x, p4.y, p4.z, p4.e};
    // index order x=0, y=1, z=2, e=3; SpinHelper's expansion equals -det[a b c d] with rows (x, y, z, e)
    double det = 0;
    const int perm[24][4] = {{0, 1, 2, 3}, {0, 1, 3, 2}, {0, 2, 1, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}, {0, 3, 2, 1},
                             {1, 0, 2, 3}, {1, 0, 3, 2}, {1, 2, 0, 3}, {1, 2, 3, 0}, {1, 3, 0, 2}, {1, 3, 2, 0},
                             {2, 0, 1, 3}, {2, 0, 3, 1}, {2, 1, 0, 3}, {2, 1, 3, 0}, {2, 3, 0, 1}, {2, 3, 1, 0},
                             {3, 0, 1, 2}, {3, 0, 2, 1}, {3, 1, 0, 2}, {3, 1, 2, 0}, {3, 2, 0, 1}, {3, 2, 1, 0}};
    for(auto &p : perm) {
        int inv = 0;
        for(int i = 0; i < 4; ++i)
            for(int j = i + 1; j < 4; ++j)
                inv += p[i] > p[j];
        const double s = (inv & 1) ? -1.0 : 1.0;
        det += s * a[p[0]] * b[p[1]] * c[p[2]] * d[p[3]];
    }
    return -det;
}
// eps_{mu nu rho sigma} a^nu b^rho c^sigma as a 4-vector (SpinHelper.h LeviCivita(a, b, c))
inline LV leviCivita3(const LV &a, const LV &b, const LV &c) {
    LV v;
    v.e = -1. * a.x * (b.y * c.z - b.z * c.y) - a.y * (b.z * c.x - b.x * c.z) - a.z * (b.x * c.y - b.y * c.x);
    v.z = a.x * (b.e * c.y - b.y * c.e) + a.y * (b.x * c.e - b.e * c.x) + a.e * (b.y * c.x - b.x * c.y);
    v.y = a.x * (b.z * c.e - b.e * c.z) + a.z * (b.e * c.x - b.x * c.e) + a.e * (b.x * c.z - b.z * c.x);
    v.x = a.y * (b.e * c.z - b.z * c.e) + a.z * (b.y * c.e - b.e * c.y) + a.e * (b.z * c.y - b.y * c.z);
    return v;
}

// get4Vecs: the four daughter 4-vectors (x, y, z, E) from the 5 variables
inline void get4Vecs(double *V, double m12, double m34, double cos12, double cos34, double phi, double M, double m1,
                     double m2, double m3, double m4) {
    double E1 = (m12 * m12 + m1 * m1 - m2 * m2) / (2 * m12);
    double E2 = (m12 * m12 - m1 * m1 + m2 * m2) / (2 * m12);
    double E3 = (m34 * m34 + m3 * m3 - m4 * m4) / (2 * m34);
    double E4 = (m34 * m34 - m3 * m3 + m4 * m4) / (2 * m34);
    double p1 = std::sqrt(E1 * E1 - m1 * m1);
    double p3 = std::sqrt(E3 * E3 - m3 * m3);
    double sin12 = std::sqrt(1 - cos12 * cos12);
    double sin34 = std::sqrt(1 - cos34 * cos34);
    double ED1 = (M * M + m12 * m12 - m34 * m34) / (2 * m12);
    double PD1 = std::sqrt(ED1 * ED1 - M * M);
    double beta1 = PD1 / ED1;
    double gamma1 = 1.0 / std::sqrt(1 - beta1 * beta1);
    double ED2 = (M * M - m12 * m12 + m34 * m34) / (2 * m34);
    double PD2 = std::sqrt(ED2 * ED2 - M * M);
    double beta2 = -PD2 / ED2;
    double gamma2 = 1.0 / std::sqrt(1 - beta2 * beta2);
    V[0] = cos12 * p1;
    V[4] = -cos12 * p1;
    V[8] = -cos34 * p3;
    V[12] = cos34 * p3;
    V[1] = sin12 * p1;
    V[5] = -sin12 * p1;
    V[9] = -sin34 * p3;
    V[13] = sin34 * p3;
    V[2] = V[6] = V[10] = V[14] = 0;
    V[3] = E1;
    V[7] = E2;
    V[11] = E3;
    V[15] = E4;
    auto boost = [&](int k, double g, double b) {
        double tE = V[4 * k + 3], tX = V[4 * k];
        V[4 * k + 3] = g * (tE + b * tX);
        V[4 * k] = g * (tX + b * tE);
    };
    boost(0, gamma1, beta1);
    boost(1, gamma1, beta1);
    boost(2, gamma2, beta2);
    boost(3, gamma2, beta2);
    double cp = std::cos(phi), sp = std::sin(phi);
    V[2] = sp * V[1];
    V[1] = cp * V[1];
    V[6] = sp * V[5];
    V[5] = cp * V[5];
}

inline double massOf(const double *a) { return std::sqrt(-a[0] * a[0] - a[1] * a[1] - a[2] * a[2] + a[3] * a[3]); }
inline double massOf(const double *a, const double *b) {
    return std::sqrt(-((a[0] + b[0]) * (a[0] + b[0])) - ((a[1] + b[1]) * (a[1] + b[1])) - ((a[2] + b[2]) * (a[2] + b[2])) +
                     ((a[3] + b[3]) * (a[3] + b[3])));
}
inline double massOf(const double *a, const double *b, const double *c) {
    return std::sqrt(-((a[0] + b[0] + c[0]) * (a[0] + b[0] + c[0])) - ((a[1] + b[1] + c[1]) * (a[1] + b[1] + c[1])) -
                     ((a[2] + b[2] + c[2]) * (a[2] + b[2] + c[2])) + ((a[3] + b[3] + c[3]) * (a[3] + b[3] + c[3])));
}

// getmass: invariant mass of a daughter combination (DP4Pair codes 2..17) and its two sub-masses
inline double getmass(unsigned pair, double &d1, double &d2, const double *V, double m1, double m2, double m3,
                      double m4) {
    const double *P1 = V, *P2 = V + 4, *P3 = V + 8, *P4 = V + 12;
    switch(pair) {
    case 2: d1 = m1; d2 = m3; return massOf(P1, P3);
    case 3: d1 = m1; d2 = m4; return massOf(P1, P4);
    case 4: d1 = m2; d2 = m3; return massOf(P2, P3);
    case 5: d1 = m2; d2 = m4; return massOf(P2, P4);
    case 6: d1 = massOf(P1, P2); d2 = m3; return massOf(P1, P2, P3);
    case 7: d1 = massOf(P1, P3); d2 = m2; return massOf(P1, P2, P3);
    case 8: d1 = massOf(P2, P3); d2 = m1; return massOf(P1, P2, P3);
    case 9: d1 = massOf(P1, P2); d2 = m4; return massOf(P1, P2, P4);
    case 10: d1 = massOf(P1, P4); d2 = m2; return massOf(P1, P2, P4);
    case 11: d1 = massOf(P2, P4); d2 = m1; return massOf(P1, P2, P4);
    case 12: d1 = massOf(P1, P3); d2 = m4; return massOf(P1, P3, P4);
    case 13: d1 = massOf(P1, P4); d2 = m3; return massOf(P1, P3, P4);
    case 14: d1 = massOf(P3, P4); d2 = m1; return massOf(P1, P3, P4);
    case 15: d1 = massOf(P2, P3); d2 = m4; return massOf(P2, P3, P4);
    case 16: d1 = massOf(P2, P4); d2 = m3; return massOf(P2, P3, P4);
    case 17: d1 = massOf(P3, P4); d2 = m2; return massOf(P2, P3, P4);
    default: d1 = d2 = 0; return 0;
    }
}

// SF_4Body kinds, numbered as the reference's enum (include/goofit/PDFs/physics/SpinFactors.h:18-35)
enum SF {
    DtoPP1_PtoSP2_StoP3P4 = 0,
    DtoPP1_PtoVP2_VtoP3P4,
    DtoV1V2_V1toP1P2_V2toP3P4_S,
    DtoV1V2_V1toP1P2_V2toP3P4_P,
    DtoV1V2_V1toP1P2_V2toP3P4_D,
    DtoAP1_AtoVP2_VtoP3P4,
    DtoAP1_AtoVP2Dwave_VtoP3P4,
    DtoVS_VtoP1P2_StoP3P4,
    DtoV1P1_V1toV2P2_V2toP3P4,
    DtoAP1_AtoSP2_StoP3P4,
    DtoTP1_TtoVP2_VtoP3P4,
    FF_12_34_L1,
    FF_12_34_L2,
    FF_123_4_L1,
    FF_123_4_L2,
    ONE
};

inline double spinFactor(int kind, double mD0, const int p[4], const double *V) {
    LV P1(V[4 * p[0]], V[4 * p[0] + 1], V[4 * p[0] + 2], V[4 * p[0] + 3]);
    LV P2(V[4 * p[1]], V[4 * p[1] + 1], V[4 * p[1] + 2], V[4 * p[1] + 3]);
    LV P3(V[4 * p[2]], V[4 * p[2] + 1], V[4 * p[2] + 2], V[4 * p[2] + 3]);
    LV P4(V[4 * p[3]], V[4 * p[3] + 1], V[4 * p[3] + 2], V[4 * p[3] + 3]);
    switch(kind) {
    case DtoPP1_PtoSP2_StoP3P4:
    case ONE: return 1.0;
    case FF_12_34_L1:
    case FF_12_34_L2:
    case FF_123_4_L1:
    case FF_123_4_L2: {
        const bool l12 = kind == FF_12_34_L1 || kind == FF_12_34_L2;
        double m1 = l12 ? (P1 + P2).mag2() : (P1 + P2 + P3).mag2();
        double m2 = l12 ? (P3 + P4).mag2() : P4.mag2();
        double s  = (P1 + P2 + P3 + P4).mag2();
        double q2 = s / 4. - (m1 + m2) / 2. + (m1 - m2) * (m1 - m2) / (4 * s);
        double z2 = q2 * mD0 * mD0;
        double ff = (kind == FF_12_34_L1 || kind == FF_123_4_L1) ? 1.0 / (1 + z2) : 1.0 / (z2 * z2 + 3 * z2 + 9);
        return std::sqrt(ff);
    }
    case DtoPP1_PtoVP2_VtoP3P4: {
        LV pV = P3 + P4, qV = P3 - P4, pP = pV + P2, qP = pV - P2;
        return zt1(qP, pP, pP.m()).dot(zt1(qV, pV, pV.m()));
    }
    case DtoV1V2_V1toP1P2_V2toP3P4_S: {
        LV pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4;
        double MV1 = std::sqrt(pV1.dot(pV1)), MV2 = std::sqrt(pV2.dot(pV2));
        return (qV1.dot(qV2) - qV1.dot(pV1) * pV1.dot(qV2) / (MV1 * MV1) - qV1.dot(pV2) * pV2.dot(qV2) / (MV2 * MV2) +
                qV1.dot(pV1) * pV1.dot(pV2) * pV2.dot(qV2) / (MV1 * MV1 * MV2 * MV2));
    }
    case DtoV1V2_V1toP1P2_V2toP3P4_P: {
        LV pV1 = P1 + P2, qV1 = P2 - P1, pV2 = P3 + P4, qV2 = P4 - P3, pD = pV1 + pV2, qD = pV1 - pV2;
        double MV1 = std::sqrt(pV1.dot(pV1)), MV2 = std::sqrt(pV2.dot(pV2));
        LV LD = zt1(qD, pD, pD.m()), LV1 = zt1(qV1, pV1, MV1), LV2 = zt1(qV2, pV2, MV2);
        return -leviCivita3(pD, LD, LV1).dot(LV2);
    }
    case DtoV1V2_V1toP1P2_V2toP3P4_D: {
        LV pV1 = P1 + P2, qV1 = P1 - P2, pV2 = P3 + P4, qV2 = P3 - P4, pD = pV1 + pV2, qD = pV1 - pV2;
        LV tV1 = zt1(qV1, pV1, pV1.m()), tV2 = zt1(qV2, pV2, pV2.m());
        T2 tD = zt2(qD, pD, pD.m());
        return tV1.dot(contract(tD, tV2));
    }
    case DtoV1P1_V1toV2P2_V2toP3P4: {
        LV pV1 = P2 + P3 + P4, pV2 = P3 + P4, qV1 = (P3 + P4) - P2, qV2 = P3 - P4;
        double MV1 = pV1.m(), MV2 = pV2.m();
        LV pD = pV1 + P1, qD = pV1 - P1;
        LV LD = zt1(qD, pD, pD.m()), LV1 = zt1(qV1, pV1, MV1), LV2 = zt1(qV2, pV2, MV2);
        LV tmp = spinSumV(pV1, MV1, LD);
        return leviCivita3(pV1, LV1, LV2).dot(tmp);
    }
    case DtoVS_VtoP1P2_StoP3P4: {
        LV pS = P3 + P4, pV = P1 + P2, qV = P1 - P2, pD = pV + pS, qD = pV - pS;
        return zt1(qD, pD, pD.m()).dot(zt1(qV, pV, pV.m()));
    }
    case DtoAP1_AtoSP2_StoP3P4: {
        LV pS = P3 + P4, pA = P2 + pS, qA = pS - P2, pD = pA + P1, qD = pA - P1;
        return zt1(qD, pD, pD.m()).dot(zt1(qA, pA, pA.m()));
    }
    case DtoAP1_AtoVP2_VtoP3P4: {
        LV pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, pD = P1 + pA, qD = pA - P1;
        LV LB = zt1(qD, pD, pD.m()), LVv = zt1(qV, pV, pV.m());
        LV tmp = spinSumV(pA, pA.m(), LVv);
        return -(LB.dot(tmp));
    }
    case DtoAP1_AtoVP2Dwave_VtoP3P4: {
        LV pV = P3 + P4, qV = P3 - P4, pA = P2 + pV, qA = P2 - pV, pD = P1 + pA, qD = pA - P1;
        LV LD = zt1(qD, pD, pD.m()), LVv = zt1(qV, pV, pV.m());
        T2 LA = zt2(qA, pA, pA.m());
        return LD.dot(contract(LA, LVv));
    }
    case DtoTP1_TtoVP2_VtoP3P4: {
        LV pV = P3 + P4, qV = P3 - P4, pT = P2 + pV, qT = pV - P2, pD = P1 + pT, qD = pT - P1;
        LV tV = zt1(qV, pV, pV.m()), tD = zt1(qD, pD, pD.m()), t1T = zt1(qT, pT, pT.m());
        LV tmp = leviCivita3(t1T, pT, spinSumV(pT, pT.m(), tV));
        return spinSumTSandwich(pT, pT.m(), tD, tD, tmp, t1T) +
               1. / 3. * tD.dot(tD) / (pT.dot(pT)) * spinSumTSandwich(pT, pT.m(), pD, pD, tmp, t1T);
    }
    default: return NAN;
    }
}

// Blatt-Weisskopf helpers (src/PDFs/physics/lineshapes/Common.cu)
inline double BL_PRIME(double z2, double z02, int L) {
    if(0 == L)
        return 1.0;
    if(1 == L)
        return (1 + z02) / (1 + z2);
    if(2 == L)
        return (z02 * z02 + 3 * z02 + 9) / (z2 * z2 + 3 * z2 + 9);
    return 0;
}
inline double BL(double z2, int L) {
    if(0 == L)
        return 1.0;
    if(1 == L)
        return 2 * z2 / (1 + z2);
    if(2 == L)
        return (13 * z2 * z2) / (z2 * z2 + 3 * z2 + 9);
    return 0;
}
inline double BL2(double z2, int L) {
    if(0 == L)
        return 1.0;
    if(1 == L)
        return 1.0 / (1 + z2);
    if(2 == L)
        return 1.0 / (z2 * z2 + 3 * z2 + 9);
    return 0;
}

// BW (RBW line shape, "ptr_to_BW_DP4") and SBW; FF codes 0 One, 1 BL, 2 BL_Prime, 3 BL2
inline std::complex<double> lineshape(bool sbw, double Mpair, double m1, double m2, double mass, double width,
                                      unsigned orbital, unsigned FF, double radius) {
    const double mumsRecoMass2 = Mpair * Mpair;
    const double mpsq = (m1 + m2) * (m1 + m2), mmsq = (m1 - m2) * (m1 - m2);
    const double num = (mumsRecoMass2 - mpsq) * (mumsRecoMass2 - mmsq);
    const double num2 = (mass * mass - mpsq) * (mass * mass - mmsq);
    const double pABSq = num / (4 * mumsRecoMass2);
    double prSq = num2 / (4 * mass * mass);
    const double prSq2 = prSq < 0 ? 0 : prSq;
    prSq = std::fabs(prSq);
    const double r2 = radius * radius;
    double frFactor = 1;
    if(0 != orbital && 0 != FF) {
        frFactor = (FF == 1 ? BL(pABSq * r2, orbital) : BL_PRIME(pABSq * r2, prSq2 * r2, orbital));
        frFactor = (FF == 3 ? BL2(pABSq * r2, orbital) : frFactor);
    }
    double GofM, k;
    if(!sbw) {
        const unsigned to2Lplus1 = 2 * orbital + 1;
        const double pratio = std::sqrt(pABSq / prSq);
        double p2j = 1;
        for(unsigned i = 0; i < to2Lplus1; i++)
            p2j *= pratio;
        const double mratio = mass / Mpair;
        const double thisFR = BL_PRIME(pABSq * r2, prSq * r2, orbital);
        GofM = width * p2j * mratio * thisFR;
        const double gamma = mass * std::sqrt((mass * mass + width * width));
        k = (2.0 * std::sqrt(2.0) / M_PI) * mass * width * gamma / std::sqrt(mass * mass + gamma);
    } else {
        GofM = width;
        const double gamma = std::sqrt(mass * mass * (mass * mass + width * width));
        k = mass * width * gamma / std::sqrt(mass * mass + gamma);
    }
    std::complex<double> bw(mass * mass - mumsRecoMass2, mass * GofM);
    const double den = (mass * mass - mumsRecoMass2) * (mass * mass - mumsRecoMass2) + mass * GofM * mass * GofM;
    return (std::sqrt(k * frFactor)) / den * bw;
}

} // namespace amp4
