// Host check of the tensor-core pass descriptors (plan.cpp: build_tc_desc) on
// random circuits: the tile geometry the kernel replays (every address in
// bounds, every entry of the state covered exactly once, every column gather
// inside the tile), every run loaded, and the BF16 operator slices: at most
// 8 significant bits each, |t_j| <= 128 units of 2^(e_row - 7 - 8j), and
// their sum equal to the operator row to 2^-47 of its largest entry.
// Prints "ok" and exits 0, or the first failure and exits 1.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "gates.h"
#include "plan.h"

using namespace dmg;

static float bf16_to_float(uint16_t b) {
  uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

template <int K>
static bool check(const PassSpec& p, int n) {
  constexpr int D = 1 << K, R = 2 * D;
  std::unique_ptr<TcDesc<K>> d(new TcDesc<K>);
  uint64_t ntiles = 0;
  int tile = 0;
  build_tc_desc(p, n, d.get(), nullptr, &ntiles, &tile);
  const PassHeader& h = d->h;
  if (h.g != 7 - K || tile != 128 * D) return std::printf("tile shape g=%d tile=%d\n", h.g, tile), false;
  const uint64_t N = 1ull << (2 * n);
  if (ntiles * (uint64_t)tile != N) return std::printf("ntiles * tile != 4^n\n"), false;
  for (int r = 0; r < (1 << h.mhi); r++)
    if (!((h.ldmask[r >> 5] >> (r & 31)) & 1)) return std::printf("run %d not loaded\n", r), false;
  // addresses of every tile (tile_base + hioff + low bits)
  std::vector<uint64_t> hioff(1 << h.mhi);
  for (int r = 0; r < (1 << h.mhi); r++) {
    uint64_t off = 0;
    for (int j = 0; j < h.mhi; j++) off |= (uint64_t)((r >> j) & 1) << h.hipos[j];
    hioff[r] = off;
  }
  std::vector<char> seen(N, 0);
  for (uint64_t t = 0; t < ntiles; t++) {
    uint64_t base = t << h.L;
    for (int j = 0; j < h.mhi; j++) {
      const int q = h.hipos[j];
      base = ((base >> q) << (q + 1)) | (base & ((1ull << q) - 1));
    }
    for (int e = 0; e < tile; e++) {
      const uint64_t ga = base + hioff[e >> h.L] + (uint64_t)(e & ((1 << h.L) - 1));
      if (ga >= N || seen[ga]) return std::printf("address %llu out of bounds or repeated\n", (unsigned long long)ga), false;
      seen[ga] = 1;
    }
  }
  // column gathers of both steps: column m = (r, f), entries lf(f) + l_r + l_c
  int lk[D], lb[D];
  for (int t = 0; t < D; t++) {
    lk[t] = lb[t] = 0;
    for (int i = 0; i < K; i++) {
      lk[t] |= ((t >> i) & 1) << h.lket[i];
      lb[t] |= ((t >> i) & 1) << h.lbra[i];
    }
  }
  std::vector<char> hit(tile, 0);
  for (int m = 0; m < 128; m++) {
    const int f = m & ((1 << h.g) - 1), r = m >> h.g;
    int lf = 0;
    for (int j = 0; j < h.g; j++) lf |= ((f >> j) & 1) << h.freepos[j];
    for (int c = 0; c < D; c++) {
      const int ket = lf + lb[r] + lk[c];
      if (ket < 0 || ket >= tile || hit[ket]) return std::printf("ket gather %d\n", ket), false;
      hit[ket] = 1;
      const int bra = lf + lk[r] + lb[c];
      if (bra < 0 || bra >= tile) return std::printf("bra gather %d\n", bra), false;
    }
  }
  // slices of the real embeddings of U (side 0) and V (side 1)
  for (int side = 0; side < 2; side++) {
    const cplx* M = side ? p.V : p.U;
    for (int row = 0; row < R; row++) {
      double w[R], mx = 0;
      for (int k = 0; k < R; k++) {
        const cplx v = M[(row % D) * D + (k % D)];
        w[k] = row < D ? (k < D ? v.real() : -v.imag()) : (k < D ? v.imag() : v.real());
        mx = std::fmax(mx, std::fabs(w[k]));
      }
      int e = 0;
      if (mx > 0) std::frexp(mx, &e);
      for (int k = 0; k < R; k++) {
        double sum = 0;
        for (int j = 0; j < kTcSlices; j++) {
          const uint32_t off = tc_kmajor_offset(row, k, 16 * R);
          if (off + 2 > (uint32_t)(R * R * 2)) return std::printf("slice offset out of range\n"), false;
          const double t = bf16_to_float(d->sl[side][j][off / 2]);
          const double units = t / std::ldexp(1.0, e - 7 - 8 * j);
          if (mx > 0 && (units != std::nearbyint(units) || std::fabs(units) > 128))
            return std::printf("slice %d of row %d: %g units\n", j, row, units), false;
          sum += t;
        }
        if (std::fabs(sum - w[k]) > std::ldexp(mx, -47)) return std::printf("row %d col %d: %g vs %g\n", row, k, sum, w[k]), false;
      }
    }
  }
  return true;
}

// complex64 descriptors: every operator entry as the sum of three BF16
// values (h, m, l), within 2^-24 of the entry rounded to FP32; slices 3..
// empty.
template <int K>
static bool check_c64(const PassSpec& p, int n) {
  constexpr int D = 1 << K, R = 2 * D;
  std::unique_ptr<TcDesc<K>> d(new TcDesc<K>);
  uint64_t ntiles = 0;
  int tile = 0;
  build_tc_desc(p, n, d.get(), nullptr, &ntiles, &tile, true, 1);
  for (int side = 0; side < 2; side++) {
    const cplx* M = side ? p.V : p.U;
    for (int row = 0; row < R; row++)
      for (int k = 0; k < R; k++) {
        const cplx v = M[(row % D) * D + (k % D)];
        const double w = row < D ? (k < D ? v.real() : -v.imag()) : (k < D ? v.imag() : v.real());
        const float wf = (float)w;
        const uint32_t off = tc_kmajor_offset(row, k, 16 * R) / 2;
        double sum = 0, prev = 1e300;
        for (int j = 0; j < kTcSlices; j++) {
          const double t = bf16_to_float(d->sl[side][j][off]);
          if (j >= 3 && t != 0) return std::printf("c64 slice %d not empty\n", j), false;
          if (j < 3 && t != 0 && std::fabs(t) > prev) return std::printf("c64 slices not decreasing\n"), false;
          if (t != 0) prev = std::fabs(t);
          sum += t;
        }
        if (std::fabs(sum - (double)wf) > std::ldexp(std::fabs((double)wf), -24))
          return std::printf("c64 row %d col %d: %.9g vs %.9g\n", row, k, sum, (double)wf), false;
      }
  }
  return true;
}

int main() {
  std::mt19937_64 rng(7);
  int checked = 0;
  for (int trial = 0; trial < 40; trial++) {
    const int n = 5 + trial % 6;  // 5..10 qubits
    std::vector<Basic> basics;
    for (int gi = 0; gi < 80; gi++) {
      GateRec g;
      std::memset(&g, 0, sizeof g);
      static const int ops[] = {0, 1, 2, 3, 8, 13, 14, 15, 16, 17, 18, 19, 20, 22, 23, 26, 27, 28, 37};
      g.op = ops[rng() % (sizeof ops / sizeof ops[0])];
      const int ar = gate_arity(g.op);
      if (ar > n) continue;
      std::vector<int> qs(n);
      for (int i = 0; i < n; i++) qs[i] = i;
      std::shuffle(qs.begin(), qs.end(), rng);
      for (int i = 0; i < ar; i++) g.qb[i] = (uint32_t)qs[i];
      std::uniform_real_distribution<double> ang(0, 6.283185307179586);
      g.theta = ang(rng);
      g.phi = ang(rng);
      g.lambda = ang(rng);
      decompose(g, basics);
    }
    for (int k : {3, 4}) {
      for (const PassSpec& p : plan_greedy(basics, k, 16)) {
        if (!tc_eligible(p, n)) continue;
        const bool ok = p.K == 3 ? (check<3>(p, n) && check_c64<3>(p, n)) : (check<4>(p, n) && check_c64<4>(p, n));
        if (!ok) return std::printf("failed: n=%d K=%d\n", n, p.K), 1;
        checked++;
      }
    }
  }
  if (checked < 100) return std::printf("too few passes checked: %d\n", checked), 1;
  std::printf("ok %d descriptors\n", checked);
  return 0;
}
