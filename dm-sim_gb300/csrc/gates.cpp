// gates.cpp -- basic-gate matrices and the composite decompositions.
//
// The matrices are the maps DM-Sim's per-gate element formulas apply to the
// ket index (src/dmsim_nvgpu_omp.cuh:1004-1481), with the trigonometric
// coefficients computed by the same expressions, so a basic gate here is the
// same operator the reference applies.  The composite sequences must be the
// reference's exactly (they define its semantics, e.g. C4X is qelib1's c4x
// transcription, not a 4-controlled X), so they follow :1493-1813 step by step.
#include "gates.h"

#include <cmath>
#include <cstring>

namespace dmg {

const char* const kOpNames[N_REF_OPS] = {
    "U3", "U2", "U1", "CX", "ID", "X", "Y", "Z", "H", "S",
    "SDG", "T", "TDG", "RX", "RY", "RZ", "CZ", "CY", "SWAP", "CH",
    "CCX", "CSWAP", "CRX", "CRY", "CRZ", "CU1", "CU3", "RXX", "RZZ", "RCCX",
    "RC3X", "C3X", "C3SQRTX", "C4X", "R", "SRN", "W", "RYY"};

namespace {

constexpr double kPi = 3.14159265358979323846;   // src/config.hpp:55
constexpr double kS2I = 0.70710678118654752440;  // src/config.hpp:57

enum RefOp {
  U3 = 0, U2, U1, CX, ID, X, Y, Z, H, S, SDG, T, TDG, RX, RY, RZ, CZ, CY, SWAP, CH,
  CCX, CSWAP, CRX, CRY, CRZ, CU1, CU3, RXX, RZZ, RCCX, RC3X, C3X, C3SQRTX, C4X, R, SRN, W, RYY
};

struct Emit {
  std::vector<Basic>& out;

  void m1(int op, int q, cplx a, cplx b, cplx c, cplx d) {
    Basic g;
    std::memset(&g, 0, sizeof g);
    g.kind = BK_1Q;
    g.op = op;
    g.q[0] = q;
    g.q[1] = -1;
    g.u[0] = a; g.u[1] = b; g.u[2] = c; g.u[3] = d;
    out.push_back(g);
  }
  // U3_GATE (:1425-1440): e0..e3 as the reference computes them
  void u3(double theta, double phi, double lambda, int q) {
    cplx e0(std::cos(theta / 2.), 0);
    cplx e1(-std::cos(lambda) * std::sin(theta / 2.), -std::sin(lambda) * std::sin(theta / 2.));
    cplx e2(std::cos(phi) * std::sin(theta / 2.), std::sin(phi) * std::sin(theta / 2.));
    cplx e3(std::cos(phi + lambda) * std::cos(theta / 2.), std::sin(phi + lambda) * std::cos(theta / 2.));
    m1(U3, q, e0, e1, e2, e3);
  }
  // U2_GATE (:1404-1418)
  void u2(double phi, double lambda, int q) {
    m1(U2, q, cplx(kS2I, 0), cplx(-kS2I * std::cos(lambda), -kS2I * std::sin(lambda)),
       cplx(kS2I * std::cos(phi), kS2I * std::sin(phi)),
       cplx(kS2I * std::cos(phi + lambda), kS2I * std::sin(phi + lambda)));
  }
  // U1_GATE (:1381-1397): diag(1, e^{i lambda})
  void u1(double lambda, int q) { m1(U1, q, 1.0, 0.0, 0.0, cplx(std::cos(lambda), std::sin(lambda))); }
  // RX_GATE (:1444-1459): [[c, i s],[i s, c]] with c = cos(t/2), s = -sin(t/2)
  void rx(double theta, int q) {
    const double c = std::cos(theta / 2.0), s = -std::sin(theta / 2.0);
    m1(RX, q, cplx(c, 0), cplx(0, s), cplx(0, s), cplx(c, 0));
  }
  // RY_GATE (:1463-1481)
  void ry(double theta, int q) {
    m1(RY, q, std::cos(theta / 2.0), -std::sin(theta / 2.0), std::sin(theta / 2.0), std::cos(theta / 2.0));
  }
  void h(int q) { m1(H, q, kS2I, kS2I, kS2I, -kS2I); }               // :1232-1245
  void x(int q) { m1(X, q, 0.0, 1.0, 1.0, 0.0); }                    // :1175-1187
  void y(int q) { m1(Y, q, 0.0, cplx(0, -1), cplx(0, 1), 0.0); }     // :1196-1209
  void z(int q) { m1(Z, q, 1.0, 0.0, 0.0, -1.0); }                   // :1216-1225
  void s(int q) { m1(S, q, 1.0, 0.0, 0.0, cplx(0, 1)); }             // :1299-1307
  void sdg(int q) { m1(SDG, q, 1.0, 0.0, 0.0, cplx(0, -1)); }        // :1314-1322
  void t(int q) { m1(T, q, 1.0, 0.0, 0.0, cplx(kS2I, kS2I)); }       // :1329-1337
  void tdg(int q) { m1(TDG, q, 1.0, 0.0, 0.0, cplx(kS2I, -kS2I)); }  // :1344-1352
  void w(int q) { m1(W, q, kS2I, cplx(0, -kS2I), cplx(0, -kS2I), kS2I); }  // :1787-1799
  void r(double p, int q) { m1(R, q, 1.0, 0.0, 0.0, cplx(0, p)); }   // :1283-1292: diag(1, i*p)
  // SRN_GATE (:1253-1266) is real-linear, not complex-linear:
  // re0' = (r0+r1)/2, im0' = (i0-i1)/2, re1' = (r0+r1)/2, im1' = (-i0+i1)/2.
  void srn(int q) {
    Basic g;
    std::memset(&g, 0, sizeof g);
    g.kind = BK_RLIN;
    g.op = SRN;
    g.q[0] = q;
    g.q[1] = -1;
    const double M[16] = {0.5, 0, 0.5, 0, 0, 0.5, 0, -0.5, 0.5, 0, 0.5, 0, 0, -0.5, 0, 0.5};
    // bra-side map: conj o M o conj, i.e. C M C with C = diag(1,-1,1,-1)
    const double C[4] = {1, -1, 1, -1};
    for (int i = 0; i < 16; i++) {
      g.rl[i] = M[i];
      g.rlb[i] = C[i / 4] * M[i] * C[i % 4];
    }
    out.push_back(g);
  }
  // CX_GATE (:1132-1168): sub-index a = bit(t) + 2 bit(c); swap a=2 <-> a=3
  void cx(int c, int tq) {
    Basic g;
    std::memset(&g, 0, sizeof g);
    g.kind = BK_2Q;
    g.op = CX;
    g.q[0] = tq;
    g.q[1] = c;
    g.u[0 * 4 + 0] = 1.0;
    g.u[1 * 4 + 1] = 1.0;
    g.u[2 * 4 + 3] = 1.0;
    g.u[3 * 4 + 2] = 1.0;
    out.push_back(g);
  }
  // CU1_GATE (:1542-1550)
  void cu1(double lambda, int a, int b) {
    u1(lambda / 2, a);
    cx(a, b);
    u1(-lambda / 2, b);
    cx(a, b);
    u1(lambda / 2, b);
  }
  // CCX_GATE (:1570-1588)
  void ccx(int a, int b, int c) {
    h(c); cx(b, c); tdg(c); cx(a, c); t(c); cx(b, c); tdg(c); cx(a, c);
    t(b); t(c); h(c); cx(a, b); t(a); tdg(b); cx(a, b);
  }
  // C3X_GATE (:1698-1728) and C3SQRTX_GATE (:1733-1763): same sequence with
  // CU1 angles of +-PI/4 and +-PI/8.
  void c3x_like(double ang, int a, int b, int c, int d) {
    h(d); cu1(-ang, a, d); h(d);
    cx(a, b);
    h(d); cu1(ang, b, d); h(d);
    cx(a, b);
    h(d); cu1(-ang, b, d); h(d);
    cx(b, c);
    h(d); cu1(ang, c, d); h(d);
    cx(a, c);
    h(d); cu1(-ang, c, d); h(d);
    cx(b, c);
    h(d); cu1(ang, c, d); h(d);
    cx(a, c);
    h(d); cu1(-ang, c, d); h(d);
  }
};

}  // namespace

int gate_arity(int op) {
  switch (op) {
    case U3: case U2: case U1: case ID: case X: case Y: case Z: case H: case S: case SDG: case T: case TDG:
    case RX: case RY: case RZ: case R: case SRN: case W: case OP_C1:
      return 1;
    case CX: case CZ: case CY: case SWAP: case CH: case CRX: case CRY: case CRZ: case CU1: case CU3:
    case RXX: case RZZ: case RYY: case OP_C2:
      return 2;
    case OP_CHANNEL:
      return 1;  // at least one; the record's nq says how many
    case CCX: case CSWAP: case RCCX:
      return 3;
    case RC3X: case C3X: case C3SQRTX:
      return 4;
    case C4X:
      return 5;
    default:
      return 0;
  }
}

void decompose(const GateRec& gr, std::vector<Basic>& out, const std::vector<Channel>* chans) {
  Emit e{out};
  const int q0 = (int)gr.qb[0], q1 = (int)gr.qb[1], q2 = (int)gr.qb[2], q3 = (int)gr.qb[3], q4 = (int)gr.qb[4];
  const double th = gr.theta, ph = gr.phi, la = gr.lambda;
  switch (gr.op) {
    case U3: e.u3(th, ph, la, q0); break;
    case U2: e.u2(ph, la, q0); break;
    case U1: e.u1(la, q0); break;
    case CX: e.cx(q0, q1); break;
    case ID: break;
    case X: e.x(q0); break;
    case Y: e.y(q0); break;
    case Z: e.z(q0); break;
    case H: e.h(q0); break;
    case S: e.s(q0); break;
    case SDG: e.sdg(q0); break;
    case T: e.t(q0); break;
    case TDG: e.tdg(q0); break;
    case RX: e.rx(th, q0); break;
    case RY: e.ry(th, q0); break;
    case RZ: e.u1(ph, q0); break;  // RZ_GATE calls U1_GATE (:1485-1489)
    // CZ (:1493-1499)
    case CZ: e.h(q1); e.cx(q0, q1); e.h(q1); break;
    // CY (:1503-1509)
    case CY: e.sdg(q1); e.cx(q0, q1); e.s(q1); break;
    // SWAP (:1591-1597)
    case SWAP: e.cx(q0, q1); e.cx(q1, q0); e.cx(q0, q1); break;
    // CH (:1513-1527)
    case CH:
      e.h(q1); e.sdg(q1); e.cx(q0, q1); e.h(q1); e.t(q1); e.cx(q0, q1); e.t(q1); e.h(q1); e.s(q1); e.x(q1); e.s(q0);
      break;
    case CCX: e.ccx(q0, q1, q2); break;
    // CSWAP (:1600-1606)
    case CSWAP: e.cx(q2, q1); e.ccx(q0, q1, q2); e.cx(q2, q1); break;
    // CRX (:1610-1618)
    case CRX:
      e.u1(kPi / 2, q1); e.cx(q0, q1); e.u3(-la / 2, 0, 0, q1); e.cx(q0, q1); e.u3(la / 2, -kPi / 2, 0, q1);
      break;
    // CRY (:1622-1629)
    case CRY: e.u3(la / 2, 0, 0, q1); e.cx(q0, q1); e.u3(-la / 2, 0, 0, q1); e.cx(q0, q1); break;
    // CRZ (:1531-1538)
    case CRZ: e.u1(la / 2, q1); e.cx(q0, q1); e.u1(-la / 2, q1); e.cx(q0, q1); break;
    case CU1: e.cu1(la, q0, q1); break;
    // CU3 (:1554-1567)
    case CU3: {
      const double temp1 = (la - ph) / 2;
      const double temp2 = th / 2;
      const double temp3 = -(ph + la) / 2;
      e.u1(-temp3, q0); e.u1(temp1, q1); e.cx(q0, q1); e.u3(-temp2, 0, temp3, q1); e.cx(q0, q1); e.u3(temp2, ph, 0, q1);
      break;
    }
    // RXX (:1633-1643)
    case RXX:
      e.u3(kPi / 2, th, 0, q0); e.h(q1); e.cx(q0, q1); e.u1(-th, q1); e.cx(q0, q1); e.h(q1); e.u2(-kPi, kPi - th, q0);
      break;
    // RZZ (:1647-1653)
    case RZZ: e.cx(q0, q1); e.u1(th, q1); e.cx(q0, q1); break;
    // RCCX (:1657-1669)
    case RCCX:
      e.u2(0, kPi, q2); e.u1(kPi / 4, q2); e.cx(q1, q2); e.u1(-kPi / 4, q2); e.cx(q0, q2); e.u1(kPi / 4, q2);
      e.cx(q1, q2); e.u1(-kPi / 4, q2); e.u2(0, kPi, q2);
      break;
    // RC3X (:1673-1694)
    case RC3X:
      e.u2(0, kPi, q3); e.u1(kPi / 4, q3); e.cx(q2, q3); e.u1(-kPi / 4, q3); e.u2(0, kPi, q3);
      e.cx(q0, q3); e.u1(kPi / 4, q3); e.cx(q1, q3); e.u1(-kPi / 4, q3); e.cx(q0, q3); e.u1(kPi / 4, q3);
      e.cx(q1, q3); e.u1(-kPi / 4, q3); e.u2(0, kPi, q3); e.u1(kPi / 4, q3); e.cx(q2, q3);
      e.u1(-kPi / 4, q3); e.u2(0, kPi, q3);
      break;
    case C3X: e.c3x_like(kPi / 4, q0, q1, q2, q3); break;
    case C3SQRTX: e.c3x_like(kPi / 8, q0, q1, q2, q3); break;
    // C4X (:1767-1780)
    case C4X:
      e.h(q4); e.cu1(-kPi / 2, q3, q4); e.h(q4);
      e.c3x_like(kPi / 4, q0, q1, q2, q3);
      e.h(q3); e.cu1(kPi / 4, q3, q4); e.h(q3);
      e.c3x_like(kPi / 4, q0, q1, q2, q3);
      e.c3x_like(kPi / 8, q0, q1, q2, q4);
      break;
    case R: e.r(th, q0); break;
    case SRN: e.srn(q0); break;
    case W: e.w(q0); break;
    // RYY (:1803-1813)
    case RYY:
      e.rx(kPi / 2, q0); e.rx(kPi / 2, q1); e.cx(q0, q1); e.u1(th, q1); e.cx(q0, q1); e.rx(-kPi / 2, q0); e.rx(-kPi / 2, q1);
      break;
    case OP_C1: {
      cplx m[4];
      for (int i = 0; i < 4; i++) m[i] = cplx(gr.m[2 * i], gr.m[2 * i + 1]);
      e.m1(OP_C1, q0, m[0], m[1], m[2], m[3]);
      break;
    }
    case OP_CHANNEL: {
      Basic g;
      std::memset(&g, 0, sizeof g);
      g.kind = BK_SUPER;
      g.op = OP_CHANNEL;
      g.q[0] = q0;
      g.q[1] = gr.nq == 2 ? q1 : -1;
      g.chan = chans ? &(*chans)[gr.chan] : nullptr;
      out.push_back(g);
      break;
    }
    case OP_C2: {
      // C2_GATE basis: pos0 = base, pos1 = +2^qubit2, pos2 = +2^qubit1, pos3 = both
      // (:1066-1069), so sub-index = bit(qubit2) + 2*bit(qubit1).
      Basic g;
      std::memset(&g, 0, sizeof g);
      g.kind = BK_2Q;
      g.op = OP_C2;
      g.q[0] = q1;
      g.q[1] = q0;
      for (int i = 0; i < 16; i++) g.u[i] = cplx(gr.m[2 * i], gr.m[2 * i + 1]);
      out.push_back(g);
      break;
    }
    default:
      break;
  }
}

}  // namespace dmg
