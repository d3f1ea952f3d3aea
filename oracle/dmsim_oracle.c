/*
 * dmsim_oracle.c -- CPU ORACLE FOR TESTS AND THE CPU BASELINE ONLY.
 *
 * A plain-C restatement of the DM-Sim CPU engine's algorithm
 * (src/dmsim_cpu_omp.hpp in pnnl/DM-Sim).  Each function cites the lines it
 * follows.  The element formulas are written with the same operand order as
 * the reference so that, compiled without FMA contraction, the results are
 * bit-identical to the reference's for a single run from |0..0><0..0|
 * (pinned by tests/test_oracle_pin.py against the reference compiled from its
 * own sources).  Not part of the product: the GPU engine never links it.
 */
#include "dmsim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constants of src/config.hpp:55-58 */
#define ORC_PI 3.14159265358979323846
#define ORC_S2I 0.70710678118654752440

/* ------------------------------------------------------------------ */
/* Basic gates: the gates the reference runs as one pass each.        */
/* ------------------------------------------------------------------ */
typedef struct {
  int op;            /* DMO_U3, DMO_U2, DMO_U1, DMO_RX, DMO_RY, DMO_X ... DMO_CX, DMO_C1, DMO_C2 */
  uint32_t q0, q1;   /* target (q0); for CX: ctrl=q0, target=q1; for C2: qubit1=q0, qubit2=q1 */
  double c[32];      /* precomputed coefficients, see basic_make() */
} basic_t;

typedef struct {
  basic_t* v;
  int n, cap;
} blist_t;

static void bl_push(blist_t* l, const basic_t* b) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 256;
    l->v = (basic_t*)realloc(l->v, sizeof(basic_t) * (size_t)l->cap);
  }
  l->v[l->n++] = *b;
}

/* Coefficients exactly as the reference computes them before the pass:
 * U3 (src/dmsim_cpu_omp.hpp:2401-2417), U2 (:2384-2399), U1 (:1395-1412),
 * RX (:1335-1352), RY (:1354-1377). */
static void b1(blist_t* l, int op, uint32_t q, double theta, double phi, double lambda) {
  basic_t b;
  memset(&b, 0, sizeof b);
  b.op = op;
  b.q0 = q;
  switch (op) {
    case DMO_U3:
      b.c[0] = cos(theta / 2.);
      b.c[1] = 0;
      b.c[2] = -cos(lambda) * sin(theta / 2.);
      b.c[3] = -sin(lambda) * sin(theta / 2.);
      b.c[4] = cos(phi) * sin(theta / 2.);
      b.c[5] = sin(phi) * sin(theta / 2.);
      b.c[6] = cos(phi + lambda) * cos(theta / 2.);
      b.c[7] = sin(phi + lambda) * cos(theta / 2.);
      b.op = DMO_C1;
      break;
    case DMO_U2:
      b.c[0] = ORC_S2I;
      b.c[1] = 0;
      b.c[2] = -ORC_S2I * cos(lambda);
      b.c[3] = -ORC_S2I * sin(lambda);
      b.c[4] = ORC_S2I * cos(phi);
      b.c[5] = ORC_S2I * sin(phi);
      b.c[6] = ORC_S2I * cos(phi + lambda);
      b.c[7] = ORC_S2I * sin(phi + lambda);
      b.op = DMO_C1;
      break;
    case DMO_U1:
      b.c[0] = cos(lambda);
      b.c[1] = sin(lambda);
      break;
    case DMO_RX:
      b.c[0] = cos(theta / 2.0);
      b.c[1] = -sin(theta / 2.0);
      break;
    case DMO_RY:
      b.c[0] = cos(theta / 2.0);
      b.c[1] = -sin(theta / 2.0);
      b.c[2] = sin(theta / 2.0);
      b.c[3] = cos(theta / 2.0);
      break;
    case DMO_R:
      b.c[0] = theta;
      break;
    default:
      break;
  }
  bl_push(l, &b);
}

static void bcx(blist_t* l, uint32_t ctrl, uint32_t tgt) {
  basic_t b;
  memset(&b, 0, sizeof b);
  b.op = DMO_CX;
  b.q0 = ctrl;
  b.q1 = tgt;
  bl_push(l, &b);
}

#define U3(t, p, la, q) b1(l, DMO_U3, (q), (t), (p), (la))
#define U2(p, la, q) b1(l, DMO_U2, (q), 0., (p), (la))
#define U1(la, q) b1(l, DMO_U1, (q), 0., 0., (la))
#define RX(t, q) b1(l, DMO_RX, (q), (t), 0., 0.)
#define RZ(p, q) b1(l, DMO_U1, (q), 0., 0., (p)) /* RZ_GATE calls U1_GATE (:2419-2423) */
#define H(q) b1(l, DMO_H, (q), 0., 0., 0.)
#define X(q) b1(l, DMO_X, (q), 0., 0., 0.)
#define S(q) b1(l, DMO_S, (q), 0., 0., 0.)
#define SDG(q) b1(l, DMO_SDG, (q), 0., 0., 0.)
#define T(q) b1(l, DMO_T, (q), 0., 0., 0.)
#define TDG(q) b1(l, DMO_TDG, (q), 0., 0., 0.)
#define CX(a, b) bcx(l, (a), (b))

/* CU1 (src/dmsim_cpu_omp.hpp:2476-2486) */
static void cu1(blist_t* l, double lambda, uint32_t a, uint32_t b) {
  U1(lambda / 2, a);
  CX(a, b);
  U1(-lambda / 2, b);
  CX(a, b);
  U1(lambda / 2, b);
}

/* CCX (src/dmsim_cpu_omp.hpp:2504-2523) */
static void ccx(blist_t* l, uint32_t a, uint32_t b, uint32_t c) {
  H(c); CX(b, c); TDG(c); CX(a, c); T(c); CX(b, c); TDG(c); CX(a, c);
  T(b); T(c); H(c); CX(a, b); T(a); TDG(b); CX(a, b);
}

/* C3X / C3SQRTX (src/dmsim_cpu_omp.hpp:2632-2699): the same sequence, with
 * CU1 angles +-PI/4 for C3X and +-PI/8 for C3SQRTX. */
static void c3x_like(blist_t* l, double ang, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  H(d); cu1(l, -ang, a, d); H(d);
  CX(a, b);
  H(d); cu1(l, ang, b, d); H(d);
  CX(a, b);
  H(d); cu1(l, -ang, b, d); H(d);
  CX(b, c);
  H(d); cu1(l, ang, c, d); H(d);
  CX(a, c);
  H(d); cu1(l, -ang, c, d); H(d);
  CX(b, c);
  H(d); cu1(l, ang, c, d); H(d);
  CX(a, c);
  H(d); cu1(l, -ang, c, d); H(d);
}

/* Decompose one gate into basic gates, following the composite definitions
 * of src/dmsim_cpu_omp.hpp:2419-2728 (identical to
 * src/dmsim_nvgpu_omp.cuh:1493-1813). */
static void decompose(blist_t* l, const dmo_gate* g) {
  const uint32_t* q = g->qb;
  const double th = g->theta, ph = g->phi, la = g->lambda;
  switch (g->op) {
    case DMO_U3: U3(th, ph, la, q[0]); break;
    case DMO_U2: U2(ph, la, q[0]); break;
    case DMO_U1: U1(la, q[0]); break;
    case DMO_CX: CX(q[0], q[1]); break;
    case DMO_ID: b1(l, DMO_ID, q[0], 0., 0., 0.); break;
    case DMO_X: X(q[0]); break;
    case DMO_Y: b1(l, DMO_Y, q[0], 0., 0., 0.); break;
    case DMO_Z: b1(l, DMO_Z, q[0], 0., 0., 0.); break;
    case DMO_H: H(q[0]); break;
    case DMO_S: S(q[0]); break;
    case DMO_SDG: SDG(q[0]); break;
    case DMO_T: T(q[0]); break;
    case DMO_TDG: TDG(q[0]); break;
    case DMO_RX: RX(th, q[0]); break;
    case DMO_RY: b1(l, DMO_RY, q[0], th, 0., 0.); break;
    case DMO_RZ: RZ(ph, q[0]); break;
    case DMO_CZ: H(q[1]); CX(q[0], q[1]); H(q[1]); break;
    case DMO_CY: SDG(q[1]); CX(q[0], q[1]); S(q[1]); break;
    case DMO_SWAP: CX(q[0], q[1]); CX(q[1], q[0]); CX(q[0], q[1]); break;
    case DMO_CH: {
      uint32_t a = q[0], b = q[1];
      H(b); SDG(b); CX(a, b); H(b); T(b); CX(a, b); T(b); H(b); S(b); X(b); S(a);
      break;
    }
    case DMO_CCX: ccx(l, q[0], q[1], q[2]); break;
    case DMO_CSWAP: CX(q[2], q[1]); ccx(l, q[0], q[1], q[2]); CX(q[2], q[1]); break;
    case DMO_CRX: {
      uint32_t a = q[0], b = q[1];
      U1(ORC_PI / 2, b); CX(a, b); U3(-la / 2, 0, 0, b); CX(a, b); U3(la / 2, -ORC_PI / 2, 0, b);
      break;
    }
    case DMO_CRY: {
      uint32_t a = q[0], b = q[1];
      U3(la / 2, 0, 0, b); CX(a, b); U3(-la / 2, 0, 0, b); CX(a, b);
      break;
    }
    case DMO_CRZ: {
      uint32_t a = q[0], b = q[1];
      U1(la / 2, b); CX(a, b); U1(-la / 2, b); CX(a, b);
      break;
    }
    case DMO_CU1: cu1(l, la, q[0], q[1]); break;
    case DMO_CU3: {
      uint32_t c = q[0], t = q[1];
      double temp1 = (la - ph) / 2;
      double temp2 = th / 2;
      double temp3 = -(ph + la) / 2;
      U1(-temp3, c); U1(temp1, t); CX(c, t); U3(-temp2, 0, temp3, t); CX(c, t); U3(temp2, ph, 0, t);
      break;
    }
    case DMO_RXX: {
      uint32_t a = q[0], b = q[1];
      U3(ORC_PI / 2, th, 0, a); H(b); CX(a, b); U1(-th, b); CX(a, b); H(b); U2(-ORC_PI, ORC_PI - th, a);
      break;
    }
    case DMO_RZZ: CX(q[0], q[1]); U1(th, q[1]); CX(q[0], q[1]); break;
    case DMO_RCCX: {
      uint32_t a = q[0], b = q[1], c = q[2];
      U2(0, ORC_PI, c); U1(ORC_PI / 4, c); CX(b, c); U1(-ORC_PI / 4, c); CX(a, c); U1(ORC_PI / 4, c);
      CX(b, c); U1(-ORC_PI / 4, c); U2(0, ORC_PI, c);
      break;
    }
    case DMO_RC3X: {
      uint32_t a = q[0], b = q[1], c = q[2], d = q[3];
      U2(0, ORC_PI, d); U1(ORC_PI / 4, d); CX(c, d); U1(-ORC_PI / 4, d); U2(0, ORC_PI, d);
      CX(a, d); U1(ORC_PI / 4, d); CX(b, d); U1(-ORC_PI / 4, d); CX(a, d); U1(ORC_PI / 4, d);
      CX(b, d); U1(-ORC_PI / 4, d); U2(0, ORC_PI, d); U1(ORC_PI / 4, d); CX(c, d);
      U1(-ORC_PI / 4, d); U2(0, ORC_PI, d);
      break;
    }
    case DMO_C3X: c3x_like(l, ORC_PI / 4, q[0], q[1], q[2], q[3]); break;
    case DMO_C3SQRTX: c3x_like(l, ORC_PI / 8, q[0], q[1], q[2], q[3]); break;
    case DMO_C4X: {
      uint32_t a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
      H(e); cu1(l, -ORC_PI / 2, d, e); H(e);
      c3x_like(l, ORC_PI / 4, a, b, c, d);
      H(d); cu1(l, ORC_PI / 4, d, e); H(d);
      c3x_like(l, ORC_PI / 4, a, b, c, d);
      c3x_like(l, ORC_PI / 8, a, b, c, e);
      break;
    }
    case DMO_R: b1(l, DMO_R, q[0], th, 0., 0.); break;
    case DMO_SRN: b1(l, DMO_SRN, q[0], 0., 0., 0.); break;
    case DMO_W: b1(l, DMO_W, q[0], 0., 0., 0.); break;
    case DMO_RYY: {
      uint32_t a = q[0], b = q[1];
      RX(ORC_PI / 2, a); RX(ORC_PI / 2, b); CX(a, b); RZ(th, b); CX(a, b); RX(-ORC_PI / 2, a); RX(-ORC_PI / 2, b);
      break;
    }
    case DMO_C1: {
      basic_t b;
      memset(&b, 0, sizeof b);
      b.op = DMO_C1;
      b.q0 = q[0];
      memcpy(b.c, g->m, 8 * sizeof(double));
      bl_push(l, &b);
      break;
    }
    case DMO_C2: {
      basic_t b;
      memset(&b, 0, sizeof b);
      b.op = DMO_C2;
      b.q0 = q[0];
      b.q1 = q[1];
      memcpy(b.c, g->m, 32 * sizeof(double));
      bl_push(l, &b);
      break;
    }
    default:
      break;
  }
}

#undef U3
#undef U2
#undef U1
#undef RX
#undef RZ
#undef H
#undef X
#undef S
#undef SDG
#undef T
#undef TDG
#undef CX

static blist_t decompose_all(const dmo_gate* gates, int ngates) {
  blist_t l = {0, 0, 0};
  for (int i = 0; i < ngates; i++) decompose(&l, &gates[i]);
  return l;
}

int dmo_basic_count(const dmo_gate* g) {
  blist_t l = decompose_all(g, 1);
  int n = l.n;
  free(l.v);
  return n;
}

/* ------------------------------------------------------------------ */
/* One basic gate on one column vector of length dim = 2^n.            */
/* Pair indexing of OP_HEAD (src/dmsim_cpu_omp.hpp:959-968) restricted */
/* to one column; element formulas of :971-1412.                       */
/* ------------------------------------------------------------------ */
static void apply_basic_vec(const basic_t* b, uint64_t dim, double* re, double* im) {
  const double S2I = ORC_S2I;
  if (b->op == DMO_CX) {
    /* CX_GATE (src/dmsim_cpu_omp.hpp:1101-1135): swap (ctrl=1,t=0) <-> (ctrl=1,t=1) */
    const uint64_t cm = (uint64_t)1 << b->q0, tm = (uint64_t)1 << b->q1;
    for (uint64_t i = 0; i < dim; i++) {
      if ((i & cm) && !(i & tm)) {
        uint64_t p0 = i, p1 = i | tm;
        double r0 = re[p0], i0 = im[p0], r1 = re[p1], i1 = im[p1];
        re[p0] = r1; im[p0] = i1; re[p1] = r0; im[p1] = i0;
      }
    }
    return;
  }
  if (b->op == DMO_C2) {
    /* C2_GATE (src/dmsim_cpu_omp.hpp:995-1094): pos0 = base, pos1 = +2^qubit2,
     * pos2 = +2^qubit1, pos3 = +both */
    const uint64_t m1 = (uint64_t)1 << b->q0, m2 = (uint64_t)1 << b->q1;
    const double* e = b->c;
    for (uint64_t i = 0; i < dim; i++) {
      if ((i & m1) || (i & m2)) continue;
      uint64_t p[4] = {i, i + m2, i + m1, i + m1 + m2};
      double r[4], m[4];
      for (int k = 0; k < 4; k++) { r[k] = re[p[k]]; m[k] = im[p[k]]; }
      for (int row = 0; row < 4; row++) {
        const double* er = e + 8 * row;
        re[p[row]] = (er[0] * r[0]) - (er[1] * m[0]) + (er[2] * r[1]) - (er[3] * m[1])
                   + (er[4] * r[2]) - (er[5] * m[2]) + (er[6] * r[3]) - (er[7] * m[3]);
        im[p[row]] = (er[0] * m[0]) + (er[1] * r[0]) + (er[2] * m[1]) + (er[3] * r[1])
                   + (er[4] * m[2]) + (er[5] * r[2]) + (er[6] * m[3]) + (er[7] * r[3]);
      }
    }
    return;
  }
  const uint32_t q = b->q0;
  const uint64_t half = dim >> 1, qm = (uint64_t)1 << q;
  const double* c = b->c;
  if (b->op == DMO_ID) return;
  for (uint64_t i = 0; i < half; i++) {
    uint64_t outer = i >> q, inner = i & (qm - 1);
    uint64_t p0 = (outer << (q + 1)) + inner, p1 = p0 + qm;
    double r0 = re[p0], i0 = im[p0], r1 = re[p1], i1 = im[p1];
    switch (b->op) {
      case DMO_C1: /* C1_GATE :971-992 */
        re[p0] = (c[0] * r0) - (c[1] * i0) + (c[2] * r1) - (c[3] * i1);
        im[p0] = (c[0] * i0) + (c[1] * r0) + (c[2] * i1) + (c[3] * r1);
        re[p1] = (c[4] * r0) - (c[5] * i0) + (c[6] * r1) - (c[7] * i1);
        im[p1] = (c[4] * i0) + (c[5] * r0) + (c[6] * i1) + (c[7] * r1);
        break;
      case DMO_U1: /* U1_GATE :1395-1412 */
        re[p0] = r0; im[p0] = i0;
        re[p1] = (c[0] * r1) - (c[1] * i1);
        im[p1] = (c[0] * i1) + (c[1] * r1);
        break;
      case DMO_RX: /* RX_GATE :1335-1352 */
        re[p0] = (c[0] * r0) - (c[1] * i1);
        im[p0] = (c[0] * i0) + (c[1] * r1);
        re[p1] = -(c[1] * i0) + (c[0] * r1);
        im[p1] = +(c[1] * r0) + (c[0] * i1);
        break;
      case DMO_RY: /* RY_GATE :1354-1377 */
        re[p0] = (c[0] * r0) + (c[1] * r1);
        im[p0] = (c[0] * i0) + (c[1] * i1);
        re[p1] = (c[2] * r0) + (c[3] * r1);
        im[p1] = (c[2] * i0) + (c[3] * i1);
        break;
      case DMO_X: /* X_GATE :1142-1154 */
        re[p0] = r1; im[p0] = i1; re[p1] = r0; im[p1] = i0;
        break;
      case DMO_Y: /* Y_GATE :1161-1175 */
        re[p0] = i1; im[p0] = -r1; re[p1] = -i0; im[p1] = r0;
        break;
      case DMO_Z: /* Z_GATE :1181-1191 */
        re[p1] = -r1; im[p1] = -i1;
        break;
      case DMO_H: /* H_GATE :1197-1211 */
        re[p0] = S2I * (r0 + r1); im[p0] = S2I * (i0 + i1);
        re[p1] = S2I * (r0 - r1); im[p1] = S2I * (i0 - i1);
        break;
      case DMO_SRN: /* SRN_GATE :1218-1232 */
        re[p0] = 0.5 * (r0 + r1); im[p0] = 0.5 * (i0 - i1);
        re[p1] = 0.5 * (r0 + r1); im[p1] = 0.5 * (-i0 + i1);
        break;
      case DMO_R: /* R_GATE :1239-1250 */
        re[p1] = -(i1 * c[0]); im[p1] = r1 * c[0];
        break;
      case DMO_S: /* S_GATE :1257-1266 */
        re[p1] = -i1; im[p1] = r1;
        break;
      case DMO_SDG: /* SDG_GATE :1272-1281 */
        re[p1] = i1; im[p1] = -r1;
        break;
      case DMO_T: /* T_GATE :1287-1296 */
        re[p1] = S2I * (r1 - i1); im[p1] = S2I * (r1 + i1);
        break;
      case DMO_TDG: /* TDG_GATE :1302-1311 */
        re[p1] = S2I * (r1 + i1); im[p1] = S2I * (-r1 + i1);
        break;
      case DMO_W: /* W_GATE :1379-1393 */
        re[p0] = S2I * (r0 + i1); im[p0] = S2I * (i0 - r1);
        re[p1] = S2I * (i0 + r1); im[p1] = S2I * (-r0 + i1);
        break;
      default:
        break;
    }
  }
}

static void apply_list_columns(int n, const blist_t* l, double* re, double* im, int nthreads) {
  const uint64_t dim = (uint64_t)1 << n;
  (void)nthreads;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t col = 0; col < (int64_t)dim; col++) {
    double* r = re + (uint64_t)col * dim;
    double* m = im + (uint64_t)col * dim;
    for (int g = 0; g < l->n; g++) apply_basic_vec(&l->v[g], dim, r, m);
  }
}

void dmo_apply_columns(int n, const dmo_gate* gates, int ngates, double* re, double* im, int nthreads) {
  blist_t l = decompose_all(gates, ngates);
  apply_list_columns(n, &l, re, im, nthreads);
  free(l.v);
}

/* conj transpose: out[a*dim+b] = conj(in[b*dim+a]); the result the
 * reference's block_transpose (src/dmsim_cpu_omp.hpp:791-825) intends. */
static void conj_transpose(uint64_t dim, const double* re, const double* im, double* ore, double* oim, int nthreads) {
  (void)nthreads;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t a = 0; a < (int64_t)dim; a++)
    for (uint64_t b = 0; b < dim; b++) {
      ore[(uint64_t)a * dim + b] = re[b * dim + (uint64_t)a];
      oim[(uint64_t)a * dim + b] = -im[b * dim + (uint64_t)a];
    }
}

void dmo_dm_sim(int n, const dmo_gate* gates, int ngates, double* re, double* im, int nthreads) {
  const uint64_t dim = (uint64_t)1 << n, N = dim * dim;
  blist_t l = decompose_all(gates, ngates);
  double* tre = (double*)malloc(N * sizeof(double));
  double* tim = (double*)malloc(N * sizeof(double));
  apply_list_columns(n, &l, re, im, nthreads);        /* forward pass */
  conj_transpose(dim, re, im, tre, tim, nthreads);     /* adjoint */
  apply_list_columns(n, &l, tre, tim, nthreads);      /* backward pass */
  memcpy(re, tre, N * sizeof(double));
  memcpy(im, tim, N * sizeof(double));
  free(tre);
  free(tim);
  free(l.v);
}

void dmo_sv_sim(int n, const dmo_gate* gates, int ngates, double* re, double* im) {
  blist_t l = decompose_all(gates, ngates);
  const uint64_t dim = (uint64_t)1 << n;
  for (int g = 0; g < l.n; g++) apply_basic_vec(&l.v[g], dim, re, im);
  free(l.v);
}

/* measure() (src/dmsim_cpu_omp.hpp:474-501; src/dmsim_nvgpu_omp.cuh:521-549) */
double dmo_measure(int n, const double* dm_re, int rep, const double* uniforms, uint64_t* out) {
  const uint64_t dim = (uint64_t)1 << n;
  double* scan = (double*)malloc((dim + 1) * sizeof(double));
  scan[0] = 0;
  for (uint64_t i = 1; i < dim + 1; i++) scan[i] = scan[i - 1] + fabs(dm_re[(i - 1) * dim + (i - 1)]);
  for (int i = 0; i < rep; i++) {
    double r = uniforms[i];
    uint64_t res = 0;
    for (uint64_t j = 0; j < dim; j++)
      if (scan[j] <= r && r < scan[j + 1]) res = j;
    out[i] = res;
  }
  double total = scan[dim];
  free(scan);
  return total;
}

void dmo_libc_uniforms(unsigned seed, int rep, double* out) {
  srand(seed);
  for (int i = 0; i < rep; i++) out[i] = (double)rand() / (double)RAND_MAX;
}
