// plan.cpp -- pass construction and the fixed-width fusion planner.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

namespace dmg {

// ---------------------------------------------------------------- fusion
namespace {

// Left-multiply the D x D group matrix U (qubit list qs) by basic gate b.
void apply_basic(cplx* U, int K, const int* qs, const Basic& b) {
  const int D = 1 << K;
  auto pos = [&](int q) {
    for (int i = 0; i < K; i++)
      if (qs[i] == q) return i;
    return -1;
  };
  if (b.kind == BK_1Q) {
    const int i = pos(b.q[0]);
    const int m = 1 << i;
    for (int c = 0; c < D; c++)
      for (int r0 = 0; r0 < D; r0++) {
        if (r0 & m) continue;
        const int r1 = r0 | m;
        const cplx x0 = U[r0 * D + c], x1 = U[r1 * D + c];
        U[r0 * D + c] = b.u[0] * x0 + b.u[1] * x1;
        U[r1 * D + c] = b.u[2] * x0 + b.u[3] * x1;
      }
  } else {  // BK_2Q: sub-index j = bit(q[0]) + 2 bit(q[1])
    const int i0 = pos(b.q[0]), i1 = pos(b.q[1]);
    const int m0 = 1 << i0, m1 = 1 << i1;
    for (int c = 0; c < D; c++)
      for (int r = 0; r < D; r++) {
        if ((r & m0) || (r & m1)) continue;
        const int rr[4] = {r, r | m0, r | m1, r | m0 | m1};
        cplx x[4];
        for (int j = 0; j < 4; j++) x[j] = U[rr[j] * D + c];
        for (int j = 0; j < 4; j++) {
          cplx acc = 0;
          for (int k = 0; k < 4; k++) acc += b.u[j * 4 + k] * x[k];
          U[rr[j] * D + c] = acc;
        }
      }
  }
}

int nq(const Basic& b) {
  if (b.kind == BK_SUPER) return b.chan->K;
  return b.kind == BK_2Q ? 2 : 1;
}

PassSpec single(const Basic& b) {
  PassSpec p;
  p.nbasic = 1;
  if (b.kind == BK_SUPER) {
    p.K = b.chan->K;
    p.q[0] = b.q[0];
    if (p.K == 2) p.q[1] = b.q[1];
    p.super = true;
    const int DD = 1 << (2 * p.K);
    for (int i = 0; i < DD * DD; i++) p.U[i] = b.chan->S[i];
    p.cls = CLS_SUPER;
    p.nnz = DD * DD;
    return p;
  }
  if (b.kind == BK_RLIN) {
    p.K = 1;
    p.q[0] = b.q[0];
    p.rlin = true;
    std::memcpy(p.rl, b.rl, sizeof p.rl);
    std::memcpy(p.rlb, b.rlb, sizeof p.rlb);
    p.cls = CLS_RLIN;
    return p;
  }
  p.K = nq(b);
  p.q[0] = b.q[0];
  if (p.K == 2) p.q[1] = b.q[1];
  const int D = 1 << p.K;
  for (int i = 0; i < D * D; i++) p.U[i] = b.u[i];
  classify(p, false);
  return p;
}

}  // namespace

std::vector<PassSpec> plan_plain(const std::vector<Basic>& basics) {
  std::vector<PassSpec> out;
  out.reserve(basics.size());
  for (const Basic& b : basics) out.push_back(single(b));
  return out;
}

std::vector<PassSpec> plan_reference_order(const std::vector<Basic>& basics) {
  std::vector<PassSpec> fwd;
  for (const Basic& b : basics) {
    PassSpec p;
    p.nbasic = 1;
    p.ket_only = true;
    if (b.kind == BK_RLIN) {
      p.K = 1;
      p.q[0] = b.q[0];
      p.rlin = true;
      std::memcpy(p.rl, b.rl, sizeof p.rl);
      for (int i = 0; i < 16; i++) p.rlb[i] = (i / 4 == i % 4) ? 1.0 : 0.0;
      p.cls = CLS_RLIN;
    } else {
      p.K = nq(b);
      p.q[0] = b.q[0];
      if (p.K == 2) p.q[1] = b.q[1];
      const int D = 1 << p.K;
      for (int i = 0; i < D * D; i++) p.U[i] = b.u[i];
      classify(p, false);
    }
    fwd.push_back(p);
  }
  std::vector<PassSpec> out = fwd;
  PassSpec t;
  t.transpose = true;
  t.K = 0;
  t.nbasic = 0;
  out.push_back(t);
  for (PassSpec& p : fwd) p.nbasic = 0;  // the second stage re-applies the same gates
  out.insert(out.end(), fwd.begin(), fwd.end());
  return out;
}

namespace {
// max nonzeros in a row of the D x D matrix U (entries below 1e-13 count as zero)
int max_row_nnz(const cplx* U, int D) {
  int mx = 0;
  for (int a = 0; a < D; a++) {
    int r = 0;
    for (int c = 0; c < D; c++) r += std::abs(U[a * D + c]) > 1e-13;
    mx = std::max(mx, r);
  }
  return mx;
}
// U (over K qubits) -> U (x) I on one more qubit (the new highest sub-index bit)
void widen(cplx* U, int K) {
  const int D = 1 << K, D2 = 2 * D;
  cplx T[kMaxD * kMaxD];
  for (int i = 0; i < D2 * D2; i++) T[i] = 0;
  for (int x = 0; x < 2; x++)
    for (int a = 0; a < D; a++)
      for (int c = 0; c < D; c++) T[(a + D * x) * D2 + (c + D * x)] = U[a * D + c];
  std::memcpy(U, T, sizeof(cplx) * D2 * D2);
}
}  // namespace

std::vector<PassSpec> plan_greedy(const std::vector<Basic>& basics, int maxk, int row_cap) {
  std::vector<PassSpec> out;
  const int m = (int)basics.size();
  if (maxk < 1) maxk = 1;
  if (maxk > kMaxK) maxk = kMaxK;
  // per-qubit program order
  int nqb = 0;
  for (const Basic& b : basics) nqb = std::max(nqb, std::max(b.q[0], b.q[1]) + 1);
  std::vector<std::vector<int>> qlist(nqb);
  for (int i = 0; i < m; i++) {
    qlist[basics[i].q[0]].push_back(i);
    if (nq(basics[i]) == 2) qlist[basics[i].q[1]].push_back(i);
  }
  std::vector<int> head(nqb, 0);
  std::vector<char> taken(m, 0);
  auto is_front = [&](int j) {
    const Basic& b = basics[j];
    if (qlist[b.q[0]][head[b.q[0]]] != j) return false;
    if (nq(b) == 2 && qlist[b.q[1]][head[b.q[1]]] != j) return false;
    return true;
  };
  auto take = [&](int j) {
    taken[j] = 1;
    head[basics[j].q[0]]++;
    if (nq(basics[j]) == 2) head[basics[j].q[1]]++;
  };
  const int kWindow = 96;  // look-ahead over untaken gates
  int first = 0;
  std::vector<int> cand;
  std::vector<char> blocked(nqb, 0);
  // Gates of the window (from the first untaken gate) that a pass holding
  // ps's qubits plus those of gate j could take, j included: a gate is
  // absorbable when all its qubits are in the set and none of them is held
  // by an earlier untaken gate that is not.
  auto absorb_count = [&](int j, const PassSpec& ps) {
    int qs[kMaxK + 2], nqs = 0;
    for (int i = 0; i < ps.K; i++) qs[nqs++] = ps.q[i];
    for (int t = 0; t < nq(basics[j]); t++) {
      bool in = false;
      for (int i = 0; i < nqs; i++) in |= qs[i] == basics[j].q[t];
      if (!in) qs[nqs++] = basics[j].q[t];
    }
    auto member = [&](int q) {
      for (int i = 0; i < nqs; i++)
        if (qs[i] == q) return true;
      return false;
    };
    std::fill(blocked.begin(), blocked.end(), 0);
    int count = 0, seen = 0;
    for (int k = first; k < m && seen < kWindow; k++) {
      if (taken[k]) continue;
      seen++;
      const Basic& b = basics[k];
      bool ok = b.kind != BK_RLIN && b.kind != BK_SUPER;
      for (int t = 0; t < nq(b); t++) ok = ok && member(b.q[t]) && !blocked[b.q[t]];
      if (ok) {
        count++;
      } else {
        for (int t = 0; t < nq(b); t++) blocked[b.q[t]] = 1;
      }
    }
    return count;
  };
  while (first < m) {
    while (first < m && taken[first]) first++;
    if (first >= m) break;
    const Basic& b0 = basics[first];
    if (b0.kind == BK_RLIN || b0.kind == BK_SUPER || nq(b0) > maxk) {  // real-linear maps and channels are barriers
      take(first);
      out.push_back(single(b0));
      continue;
    }
    PassSpec p;
    p.K = 0;
    p.U[0] = 1.0;
    auto add_qubit = [&](PassSpec& ps, int q) {
      for (int i = 0; i < ps.K; i++)
        if (ps.q[i] == q) return;
      widen(ps.U, ps.K);
      ps.q[ps.K++] = q;
    };
    add_qubit(p, b0.q[0]);
    if (nq(b0) == 2) add_qubit(p, b0.q[1]);
    apply_basic(p.U, p.K, p.q, b0);
    take(first);
    int members = 1;
    for (;;) {
      // candidates in preference order: fewest new qubits, then program order
      cand.clear();
      int seen = 0;
      for (int j = first + 1; j < m && seen < kWindow; j++) {
        if (taken[j]) continue;
        seen++;
        const Basic& b = basics[j];
        if (b.kind == BK_RLIN || b.kind == BK_SUPER || !is_front(j)) continue;
        int add = 0;
        for (int t = 0; t < nq(b); t++) {
          bool in = false;
          for (int i = 0; i < p.K; i++) in |= p.q[i] == b.q[t];
          add += in ? 0 : 1;
        }
        if (p.K + add > maxk) continue;
        cand.push_back(add * m + j);
      }
      if (cand.empty()) break;
      std::sort(cand.begin(), cand.end());
      // When every candidate widens the pass, the qubit it brings decides
      // which later gates the pass can still take: rank those candidates by
      // how many gates of the window the widened qubit set would absorb
      // (program order on every qubit respected), most first, then by the
      // order above.
      if (cand.front() / m > 0 && p.K < maxk) {
        std::vector<std::pair<int, int>> ranked;  // (-absorbed, key)
        ranked.reserve(cand.size());
        for (int key : cand) ranked.push_back({-absorb_count(key % m, p), key});
        std::stable_sort(ranked.begin(), ranked.end());
        for (size_t i = 0; i < cand.size(); i++) cand[i] = ranked[i].second;
      }
      bool grown = false;
      for (int key : cand) {
        const int j = key % m;
        PassSpec trial = p;
        const Basic& b = basics[j];
        add_qubit(trial, b.q[0]);
        if (nq(b) == 2) add_qubit(trial, b.q[1]);
        apply_basic(trial.U, trial.K, trial.q, b);
        if (row_cap < kMaxD && max_row_nnz(trial.U, 1 << trial.K) > row_cap) continue;
        p = trial;
        take(j);
        members++;
        grown = true;
        break;
      }
      if (!grown) break;
    }
    if (members == 1) {
      out.push_back(single(b0));
      continue;
    }
    p.nbasic = members;
    classify(p, true);
    out.push_back(p);
  }
  return out;
}

// ---------------------------------------------------------------- classes
namespace {
// Entries within this distance of 0, +-1 are taken as exact.  Products of
// up to a few hundred basic gates carry roundoff of order 1e-15; a fused
// operator's structural zeros and ones are restored exactly so the kernel
// can skip the arithmetic.
constexpr double kSnapFused = 1e-13;
// For a single basic gate only the superoperator factors are snapped (e.g.
// |T11|^2 = 1 + 2e-16); the matrix entries are taken as given.
constexpr double kSnapFactor = 1e-15;

double snap1(double x, double eps) {
  if (std::fabs(x) < eps) return 0.0;
  if (std::fabs(x - 1.0) < eps) return 1.0;
  if (std::fabs(x + 1.0) < eps) return -1.0;
  return x;
}
}  // namespace

void classify(PassSpec& p, bool fused) {
  if (p.super) {
    p.cls = CLS_SUPER;
    return;
  }
  if (p.rlin) {
    p.cls = CLS_RLIN;
    p.nnz = 4;
    return;
  }
  const int D = 1 << p.K;
  if (fused)
    for (int i = 0; i < D * D; i++) p.U[i] = cplx(snap1(p.U[i].real(), kSnapFused), snap1(p.U[i].imag(), kSnapFused));
  for (int i = 0; i < D * D; i++) p.V[i] = p.ket_only ? cplx(i / D == i % D ? 1.0 : 0.0, 0.0) : std::conj(p.U[i]);
  auto count = [&](const cplx* M, bool& mono) {
    int nnz = 0;
    mono = true;
    std::vector<int> colcount(D, 0);
    for (int a = 0; a < D; a++) {
      int rn = 0;
      for (int c = 0; c < D; c++)
        if (M[a * D + c] != cplx(0, 0)) {
          rn++;
          colcount[c]++;
        }
      nnz += rn;
      if (rn != 1) mono = false;
    }
    for (int c = 0; c < D; c++)
      if (colcount[c] != 1) mono = false;
    return nnz;
  };
  bool mono_u, mono_v;
  const int nnz = count(p.U, mono_u);
  count(p.V, mono_v);
  p.nnz = nnz;
  if (mono_u && mono_v) {
    bool all_one = true, all_signed = true;
    for (int a = 0; a < D; a++) {
      int sa = 0;
      while (p.U[a * D + sa] == cplx(0, 0)) sa++;
      for (int b = 0; b < D; b++) {
        int sb = 0;
        while (p.V[b * D + sb] == cplx(0, 0)) sb++;
        const cplx f = p.U[a * D + sa] * p.V[b * D + sb];
        const double fr = snap1(f.real(), kSnapFactor), fi = snap1(f.imag(), kSnapFactor);
        const bool one = fr == 1.0 && fi == 0.0;
        const bool sgn = one || (fr == -1.0 && fi == 0.0) || (fr == 0.0 && (fi == 1.0 || fi == -1.0));
        all_one &= one;
        all_signed &= sgn;
      }
    }
    p.cls = all_one ? CLS_MOVE : (all_signed ? CLS_SIGNED : CLS_PHASE);
    return;
  }
  p.cls = (4 * nnz > 3 * D * D) ? CLS_DENSE : CLS_SPARSE;
}

// ---------------------------------------------------------------- descriptors
size_t desc_size(int K) {
  switch (K) {
    case 1: return sizeof(PassDesc<1>);
    case 2: return sizeof(PassDesc<2>);
    case 3: return sizeof(PassDesc<3>);
    default: return sizeof(PassDesc<4>);
  }
}

namespace {

template <int K>
uint64_t build_k(const PassSpec& p, int n, PassDesc<K>* d, PassFeatures* feat, uint64_t* ntiles_out, int* tile_out,
                 int g_cap) {
  constexpr int D = 1 << K;
  std::memset(d, 0, sizeof(*d));
  PassHeader& h = d->h;
  PassOp<K>& op = d->op;
  const int nb = 2 * n;
  h.K = K;
  h.cls = p.cls;
  // target bit positions
  std::vector<int> P;
  for (int i = 0; i < K; i++) {
    P.push_back(p.q[i]);
    P.push_back(p.q[i] + n);
  }
  std::sort(P.begin(), P.end());
  std::vector<int> F;
  for (int b = 0; b < nb; b++)
    if (!std::binary_search(P.begin(), P.end(), b)) F.push_back(b);
  // at least one free bit in the low run keeps runs >= 2 entries long (the
  // kernels move entries in 16-byte pairs)
  int g = std::min(8 - K, std::max(g_cap, 1));
  if (g > (int)F.size()) g = (int)F.size();
  // L: the position of the (g+1)-th free bit, so that exactly g free bits
  // and every target bit below it lie in the contiguous low run.
  const int L = (g < (int)F.size()) ? F[g] : nb;
  std::vector<int> hi;
  for (int x : P)
    if (x >= L) hi.push_back(x);
  h.g = g;
  h.L = L;
  h.mhi = (int)hi.size();
  for (int j = 0; j < h.mhi; j++) h.hipos[j] = hi[j];
  auto local = [&](int x) {
    if (x < L) return x;
    return L + (int)(std::lower_bound(hi.begin(), hi.end(), x) - hi.begin());
  };
  for (int i = 0; i < K; i++) {
    h.lket[i] = local(p.q[i]);
    h.lbra[i] = local(p.q[i] + n);
  }
  for (int j = 0; j < g; j++) h.freepos[j] = F[j];
  h.ntiles = 1ull << (nb - L - h.mhi);

  // operator tables
  bool real = p.cls == CLS_DENSE || p.cls == CLS_SPARSE;
  for (int i = 0; i < D * D; i++) {
    op.ure[i] = p.U[i].real();
    op.uim[i] = p.U[i].imag();
    op.vre[i] = p.V[i].real();
    op.vim[i] = p.V[i].imag();
    real = real && op.uim[i] == 0.0 && op.vim[i] == 0.0;
  }
  if (real) h.flags |= kPassRealOperator;
  std::memcpy(op.rlin, p.rl, sizeof op.rlin);
  std::memcpy(op.rlinb, p.rlb, sizeof op.rlinb);
  if (p.cls == CLS_SUPER && K <= 2) {
    for (int i = 0; i < D * D * D * D; i++) {
      op.sre[i] = p.U[i].real();
      op.sim[i] = p.U[i].imag();
    }
  }
  int src[kMaxD], srcb[kMaxD];
  for (int a = 0; a < D; a++) {
    int j = 0;
    for (int c = 0; c < D; c++)
      if (p.U[a * D + c] != cplx(0, 0)) op.col[a * D + j++] = (int8_t)c;
    op.nnz[a] = (int8_t)j;
    src[a] = j > 0 ? op.col[a * D] : a;
    op.src[a] = (int8_t)src[a];
    int jb = 0;
    for (int c = 0; c < D; c++)
      if (p.V[a * D + c] != cplx(0, 0)) op.colb[a * D + jb++] = (int8_t)c;
    op.nnzb[a] = (int8_t)jb;
    srcb[a] = jb > 0 ? op.colb[a * D] : a;
    op.srcb[a] = (int8_t)srcb[a];
    op.nnzmax = std::max<int8_t>(op.nnzmax, op.nnz[a]);
    op.nnzbmax = std::max<int8_t>(op.nnzbmax, op.nnzb[a]);
  }
  const bool mono = p.cls == CLS_MOVE || p.cls == CLS_SIGNED || p.cls == CLS_PHASE;
  for (int a = 0; a < D; a++)
    for (int b = 0; b < D; b++) {
      int8_t fk = FK_GEN;
      if (mono) {
        const cplx f = p.U[a * D + src[a]] * p.V[b * D + srcb[b]];
        const double fr = snap1(f.real(), kSnapFactor), fi = snap1(f.imag(), kSnapFactor);
        op.fre[a * D + b] = fr;
        op.fim[a * D + b] = fi;
        if (fr == 1.0 && fi == 0.0) fk = FK_ONE;
        else if (fr == -1.0 && fi == 0.0) fk = FK_NEG;
        else if (fr == 0.0 && fi == 1.0) fk = FK_PI;
        else if (fr == 0.0 && fi == -1.0) fk = FK_NI;
      }
      op.fk[a * D + b] = fk;
    }

  // run masks
  auto run_of = [&](int a, int b) {
    int r = 0;
    for (int j = 0; j < h.mhi; j++) {
      const int x = hi[j];
      int bit = 0;
      for (int i = 0; i < K; i++) {
        if (x == p.q[i]) bit = (a >> i) & 1;
        if (x == p.q[i] + n) bit = (b >> i) & 1;
      }
      r |= bit << j;
    }
    return r;
  };
  auto row_identity = [&](const cplx* M, int a) {
    for (int c = 0; c < D; c++)
      if (M[a * D + c] != (c == a ? cplx(1, 0) : cplx(0, 0))) return false;
    return true;
  };
  std::vector<char> st(1 << h.mhi, 0), ld(1 << h.mhi, 0);
  for (int a = 0; a < D; a++)
    for (int b = 0; b < D; b++) {
      bool changed;
      if (p.cls == CLS_RLIN || p.cls == CLS_SUPER) changed = true;
      else if (mono) changed = src[a] != a || srcb[b] != b || op.fk[a * D + b] != FK_ONE;
      else changed = !(row_identity(p.U, a) && row_identity(p.V, b));
      if (changed) st[run_of(a, b)] = 1;
    }
  for (int a = 0; a < D; a++)
    for (int b = 0; b < D; b++) {
      if (!st[run_of(a, b)]) continue;
      ld[run_of(a, b)] = 1;
      if (p.cls == CLS_RLIN || p.cls == CLS_SUPER) {
        for (int a2 = 0; a2 < D; a2++)
          for (int b2 = 0; b2 < D; b2++) ld[run_of(a2, b2)] = 1;
      } else if (mono) {
        ld[run_of(src[a], srcb[b])] = 1;
      } else {
        for (int c = 0; c < D; c++) {
          if (p.U[a * D + c] == cplx(0, 0)) continue;
          for (int e = 0; e < D; e++)
            if (p.V[b * D + e] != cplx(0, 0)) ld[run_of(c, e)] = 1;
        }
      }
    }
  // DENSE and RLIN multiply every entry of a column, structural zeros
  // included, so every run is loaded: an unloaded run would feed
  // uninitialised shared memory (possibly NaN, and 0*NaN = NaN) into stored
  // entries.  MOVE/SIGNED/PHASE/SPARSE read only the sources listed above.
  if (p.cls == CLS_DENSE || p.cls == CLS_RLIN || p.cls == CLS_SUPER) std::fill(ld.begin(), ld.end(), 1);
  int nst = 0, nld = 0;
  for (int r = 0; r < (1 << h.mhi); r++) {
    if (st[r]) {
      h.stmask[r >> 5] |= 1u << (r & 31);
      nst++;
    }
    if (ld[r]) {
      h.ldmask[r >> 5] |= 1u << (r & 31);
      nld++;
    }
  }
  const uint64_t runlen = 1ull << L;
  const uint64_t entries = (uint64_t)(nst + nld) * runlen * h.ntiles;
  if (ntiles_out) *ntiles_out = h.ntiles;
  if (tile_out) *tile_out = (1 << g) * D * D;
  if (feat) {
    feat->K = K;
    feat->cls = p.cls;
    feat->nnz = p.nnz;
    feat->real = real ? 1 : 0;
    feat->n = n;
    int lo = -1, hmin = nb;
    for (int x : P) {
      if (x < L) lo = std::max(lo, x);
      else hmin = std::min(hmin, x);
    }
    feat->max_lo_bit = lo;
    feat->min_hi_bit = hmin;
    const double tot = (double)(1 << h.mhi);
    feat->ld_frac = nld / tot;
    feat->st_frac = nst / tot;
  }
  return entries;
}

}  // namespace

// Tensor-core pass: the geometry of the K-qubit pass with 2^(7-K) groups per
// tile (128 columns per step), every run loaded, and the BF16 slices of the
// real embeddings of U (ket) and V (bra).
// x rounded to the nearest BF16 value (8 significant bits, ties to even), as
// a float.
float bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return x;  // inf / nan: unchanged
  u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

template <int K>
uint64_t build_tc_k(const PassSpec& p, int n, TcDesc<K>* d, PassFeatures* feat, uint64_t* ntiles_out,
                    int* tile_out, bool slices, bool per_entry) {
  constexpr int D = 1 << K, R = 2 * D;
  std::unique_ptr<PassDesc<K>> geo(new PassDesc<K>);
  build_k<K>(p, n, geo.get(), feat, ntiles_out, tile_out, 7 - K);
  std::memset(d, 0, sizeof(*d));
  d->h = geo->h;
  PassHeader& h = d->h;
  const int nruns = 1 << h.mhi;
  int nst = 0;
  for (int r = 0; r < nruns; r++) {
    h.ldmask[r >> 5] |= 1u << (r & 31);
    nst += (h.stmask[r >> 5] >> (r & 31)) & 1;
  }
  if (feat) feat->ld_frac = 1.0;
  for (int side = 0; side < 2 && slices; side++) {
    const cplx* M = side ? p.V : p.U;
    for (int row = 0; row < R; row++) {
      double w[R];
      const int a = row % D;
      for (int k = 0; k < R; k++) {
        const cplx m = M[a * D + (k % D)];
        if (row < D) w[k] = k < D ? m.real() : -m.imag();
        else w[k] = k < D ? m.imag() : m.real();
      }
      if (per_entry) {
        // complex64 state: each entry of the FP32-rounded operator as the sum
        // of three BF16 values (hi, mid, lo), each rounded from the remainder
        // of the ones before it
        for (int k = 0; k < R; k++) {
          float v = (float)w[k];
          for (int j = 0; j < kTcSlices; j++) {
            uint32_t bits = 0;
            if (j < 3) {
              const float t = bf16_round(v);
              std::memcpy(&bits, &t, 4);
              v -= t;  // exact: the remainder of a rounding to 8 significant bits
            }
            d->sl[side][j][tc_kmajor_offset(row, k, 16 * R) / 2] = (uint16_t)(bits >> 16);
          }
        }
        continue;
      }
      double mx = 0;
      for (int k = 0; k < R; k++) mx = std::max(mx, std::fabs(w[k]));
      int e = 0;
      if (mx > 0) std::frexp(mx, &e);  // mx in [2^(e-1), 2^e)
      for (int k = 0; k < R; k++) {
        double v = w[k];
        for (int j = 0; j < kTcSlices; j++) {
          const double unit = std::ldexp(1.0, e - 7 - 8 * j);
          const double t = mx > 0 ? std::nearbyint(v / unit) * unit : 0.0;  // |t| <= 128 units: exact in BF16
          const float tf = (float)t;
          uint32_t bits;
          std::memcpy(&bits, &tf, 4);
          d->sl[side][j][tc_kmajor_offset(row, k, 16 * R) / 2] = (uint16_t)(bits >> 16);
          v -= t;
        }
      }
    }
  }
  const uint64_t runlen = 1ull << h.L;
  return (uint64_t)(nst + nruns) * runlen * h.ntiles;
}

void tc64_digits(int64_t t, int d[7]) {
  // u = t + 0x80 in every byte: each byte of u minus 0x80 is a balanced digit
  const uint64_t u = (uint64_t)t + 0x0080808080808080ull;
  for (int j = 1; j < 7; j++) d[j] = (int)((u >> (8 * (6 - j))) & 0xFF) - 128;
  d[0] = (int)(u >> 48) - 128;
}

// The FP64-width descriptor: the geometry of the double-float tensor pass and
// the operator's rows as 56-bit integers times a power of two, in digits.
template <int K>
uint64_t build_tc64_k(const PassSpec& p, int n, TcDesc64<K>* d, PassFeatures* feat, uint64_t* ntiles_out,
                      int* tile_out, bool slices) {
  constexpr int D = 1 << K, R = 2 * D;
  std::unique_ptr<PassDesc<K>> geo(new PassDesc<K>);
  build_k<K>(p, n, geo.get(), feat, ntiles_out, tile_out, 7 - K);
  std::memset(d, 0, sizeof(*d));
  d->h = geo->h;
  PassHeader& h = d->h;
  const int nruns = 1 << h.mhi;
  int nst = 0;
  for (int r = 0; r < nruns; r++) {
    h.ldmask[r >> 5] |= 1u << (r & 31);
    nst += (h.stmask[r >> 5] >> (r & 31)) & 1;
  }
  if (feat) feat->ld_frac = 1.0;
  for (int side = 0; side < 2 && slices; side++) {
    const cplx* M = side ? p.V : p.U;
    for (int a = 0; a < D; a++) {
      // rows a ([Ur, -Ui]) and a + D ([Ui, Ur]) hold the same magnitudes
      double mx = 0;
      for (int k = 0; k < D; k++) mx = std::max(mx, std::max(std::fabs(M[a * D + k].real()), std::fabs(M[a * D + k].imag())));
      int e = 0;
      if (mx > 0) std::frexp(mx, &e);  // every |entry| < 2^e
      d->ew[side][a] = mx > 0 ? e - 55 : 0;
      for (int half = 0; half < 2; half++) {
        const int row = a + half * D;
        for (int k = 0; k < R; k++) {
          const cplx m = M[a * D + (k % D)];
          const double w = half == 0 ? (k < D ? m.real() : -m.imag()) : (k < D ? m.imag() : m.real());
          const int64_t t = mx > 0 ? (int64_t)std::nearbyint(std::ldexp(w, 55 - e)) : 0;  // |t| <= 2^55
          int dg[7];
          tc64_digits(t, dg);
          for (int j = 0; j < kTc64Slices; j++) {
            const float tf = (float)dg[j];  // |digit| <= 128: exact in BF16
            uint32_t bits;
            std::memcpy(&bits, &tf, 4);
            d->sl[side][j][tc_kmajor_offset(row, k, 16 * R) / 2] = (uint16_t)(bits >> 16);
          }
        }
      }
    }
  }
  const uint64_t runlen = 1ull << h.L;
  return (uint64_t)(nst + nruns) * runlen * h.ntiles;
}

uint64_t build_tc_desc(const PassSpec& p, int n, void* out, PassFeatures* f, uint64_t* ntiles, int* tile_entries,
                       bool slices, int arith) {
  if (arith == 0) {
    if (p.K == 3) return build_tc64_k<3>(p, n, static_cast<TcDesc64<3>*>(out), f, ntiles, tile_entries, slices);
    return build_tc64_k<4>(p, n, static_cast<TcDesc64<4>*>(out), f, ntiles, tile_entries, slices);
  }
  // complex64 (arith 1): per-entry BF16 x 3 slices (tensor32.cu); double-float:
  // 6 slices on per-row grids (tensor.cu)
  const bool per_entry = arith == 1;
  if (p.K == 3) return build_tc_k<3>(p, n, static_cast<TcDesc<3>*>(out), f, ntiles, tile_entries, slices, per_entry);
  return build_tc_k<4>(p, n, static_cast<TcDesc<4>*>(out), f, ntiles, tile_entries, slices, per_entry);
}

bool tc_eligible(const PassSpec& p, int n) {
  if (p.transpose || p.rlin || p.super) return false;
  if (p.K != 3 && p.K != 4) return false;
  if (p.cls != CLS_DENSE && p.cls != CLS_SPARSE) return false;
  // 7 - K free bits must fit below the tile: 2n - 2K >= 7 - K
  return 2 * n - 2 * p.K >= 7 - p.K;
}

bool tc_choose(const PassSpec& p, int n, int tensor_opt, int arith) {
  if (!tensor_opt || !tc_eligible(p, n)) return false;
  if (tensor_opt == 2) return true;  // every eligible pass (measurements)
  if (p.tc >= 0) return p.tc != 0;   // the learned planner's choice
  if (arith == 0) return true;       // FP64: the alternative is GB300's FP64 pipe
  // complex64: 4-qubit passes on the tensor cores (tensor32.cu: 2530 against
  // 1790 GB/s for the FP32-pipe kernel at 14 qubits); 3-qubit ones stay on the
  // FP32 pipe (2820 against 2360 GB/s)
  if (arith == 1) return p.K == 4;
  return p.nnz >= kTcMinRowNnz * (1 << p.K);
}

size_t tc_desc_bytes(int K, int arith) {
  if (arith == 0) return K == 3 ? sizeof(TcDesc64<3>) : sizeof(TcDesc64<4>);
  return K == 3 ? sizeof(TcDesc<3>) : sizeof(TcDesc<4>);
}

uint64_t build_desc(const PassSpec& p, int n, void* out, PassFeatures* f, uint64_t* ntiles, int* tile_entries,
                    int g_cap) {
  switch (p.K) {
    case 1: return build_k<1>(p, n, static_cast<PassDesc<1>*>(out), f, ntiles, tile_entries, g_cap);
    case 2: return build_k<2>(p, n, static_cast<PassDesc<2>*>(out), f, ntiles, tile_entries, g_cap);
    case 3: return build_k<3>(p, n, static_cast<PassDesc<3>*>(out), f, ntiles, tile_entries, g_cap);
    default: return build_k<4>(p, n, static_cast<PassDesc<4>*>(out), f, ntiles, tile_entries, g_cap);
  }
}

}  // namespace dmg
