// Host-side check of the engine's gate fusion (qgb_fuse5 in qgb_fuse.cu).
//
// Random gate lists (dense 1- and 2-qubit gates, controlled gates with up to
// 3 controls, diagonal gates with and without entries equal to 1, gates
// spanning more than 5 qubits that must stay unfused) are
// applied to random states of 6..10 qubits gate by gate and as the fused list
// (every other case with padding to 5-qubit blocks);
// the results must agree to 1e-12.  Fused ops must be uncontrolled and act on
// at most 5 qubits unless they are an original gate.  Also prints the block
// count of the 30-qubit, depth-20 U3 + CZ brickwork (all blocks should be
// 5-qubit blocks but the last few).  No kernel is launched.
#include <complex>
#include <cstdio>
#include <random>

#include "qgb_fuse.cu"

typedef std::complex<double> cd;

// apply op (qibo order: qubit q is index bit n-1-q; controls must be 1)
static void apply(std::vector<cd>& psi, int n, const qgb_op& op, const double* m) {
  const int k = op.k, dk = 1 << k;
  long long tmask = 0, cmask = 0;
  int tb[5];
  for (int j = 0; j < k; ++j) {
    tb[j] = n - 1 - op.qubits[j];
    tmask |= 1ll << tb[j];
  }
  for (int j = 0; j < op.ncontrols; ++j) cmask |= 1ll << (n - 1 - op.controls[j]);
  const long long N = 1ll << n;
  for (long long base = 0; base < N; ++base) {
    if ((base & tmask) || (base & cmask) != cmask) continue;
    long long idx[32];
    cd in[32];
    for (int a = 0; a < dk; ++a) {
      long long i = base;
      for (int j = 0; j < k; ++j)
        if ((a >> (k - 1 - j)) & 1) i |= 1ll << tb[j];
      idx[a] = i;
      in[a] = psi[i];
    }
    for (int r = 0; r < dk; ++r) {
      cd acc = 0;
      for (int a = 0; a < dk; ++a) acc += cd(m[2 * (r * dk + a)], m[2 * (r * dk + a) + 1]) * in[a];
      psi[idx[r]] = acc;
    }
  }
}

int main() {
  std::mt19937_64 rng(21);
  std::normal_distribution<double> nd;
  int fails = 0;
  double worst = 0;
  for (int trial = 0; trial < 60; ++trial) {
    const int n = 6 + trial % 5;
    std::vector<qgb_op> ops;
    std::vector<double> coefs;
    const int ngates = 20 + (int)(rng() % 60);
    for (int i = 0; i < ngates; ++i) {
      qgb_op o = qgb_op();
      std::vector<int> q(n);
      for (int j = 0; j < n; ++j) q[j] = j;
      std::shuffle(q.begin(), q.end(), rng);
      const int kind = (int)(rng() % 13);
      o.k = kind < 5 || kind == 10 || kind == 11 ? 1 : 2;
      o.ncontrols = kind == 8 || kind == 11 ? 1 + (int)(rng() % 3) : kind == 12 ? (int)(rng() % 2) : 0;
      if (kind == 9) {  // a gate on more than 5 qubits: 2 targets, 4 controls
        o.k = 2;
        o.ncontrols = std::min(4, n - 2);
      }
      for (int j = 0; j < o.k; ++j) o.qubits[j] = q[j];
      for (int j = 0; j < o.ncontrols; ++j) o.controls[j] = q[o.k + j];
      o.coef_offset = (int64_t)coefs.size();
      const int d = 1 << o.k;
      for (int e = 0; e < d * d; ++e) {
        double re = nd(rng), im = nd(rng);
        if ((kind == 7 || kind == 10 || kind == 12) && (e / d != e % d)) re = im = 0;  // diagonal gates too
        if (kind == 10 && e == 0) re = 1.0 / 0.3, im = 0;  // a phase gate: entry (0, 0) exactly 1
        if (kind == 12 && e / d == e % d) re = (e == d * d - 1 ? -1.0 : 1.0) / 0.3, im = 0;  // CZ, maybe controlled
        coefs.push_back(0.3 * re);
        coefs.push_back(0.3 * im);
      }
      ops.push_back(o);
    }
    const long long N = 1ll << n;
    std::vector<cd> a(N), b;
    for (auto& x : a) x = cd(nd(rng), nd(rng));
    b = a;
    for (const qgb_op& o : ops) apply(a, n, o, coefs.data() + o.coef_offset);
    std::vector<qgb_op> fo;
    std::vector<double> fc;
    qgb_fuse5(ops.data(), (int)ops.size(), coefs.data(), &fo, &fc, trial % 2 ? n : 0);
    bool bad = false;
    for (const qgb_op& o : fo) {
      if (trial % 2 && o.k + o.ncontrols <= 5 && o.k != 5) bad = true;  // padded: every fusable op on 5 qubits
      if (o.k + o.ncontrols > 5) {  // must be one of the original wide gates
        bool found = false;
        for (const qgb_op& p : ops)
          found = found || (p.k == o.k && p.ncontrols == o.ncontrols && p.qubits[0] == o.qubits[0] &&
                            p.controls[0] == o.controls[0]);
        bad = bad || !found;
      }
      apply(b, n, o, fc.data() + o.coef_offset);
    }
    double err = 0, nrm = 0;
    for (long long i = 0; i < N; ++i) {
      err = std::max(err, std::abs(a[i] - b[i]));
      nrm = std::max(nrm, std::abs(a[i]));
    }
    worst = std::max(worst, err / nrm);
    if (bad || err > 1e-12 * nrm) {
      ++fails;
      printf("FAIL trial %d n=%d gates %d -> %zu ops, rel err %g bad %d\n", trial, n, ngates, fo.size(), err / nrm,
             (int)bad);
    }
  }
  // the 30-qubit depth-20 brickwork: U3 on every qubit, then CZ on pairs
  {
    const int n = 30;
    std::vector<qgb_op> ops;
    std::vector<double> coefs;
    for (int l = 0; l < 20; ++l) {
      for (int q = 0; q < n; ++q) {
        qgb_op o = qgb_op();
        o.k = 1;
        o.qubits[0] = q;
        o.coef_offset = (int64_t)coefs.size();
        for (int e = 0; e < 8; ++e) coefs.push_back(nd(rng));
        ops.push_back(o);
      }
      for (int q = l % 2; q + 1 < n; q += 2) {
        qgb_op o = qgb_op();
        o.k = 2;
        o.qubits[0] = q;
        o.qubits[1] = q + 1;
        o.coef_offset = (int64_t)coefs.size();
        for (int e = 0; e < 16; ++e) coefs.push_back(e == 0 || e == 10 || e == 20 ? 1.0 : e == 30 ? -1.0 : 0.0);
        ops.push_back(o);
      }
    }
    std::vector<qgb_op> fo;
    std::vector<double> fc;
    qgb_fuse5(ops.data(), (int)ops.size(), coefs.data(), &fo, &fc, 0);
    int n5 = 0;
    for (const qgb_op& o : fo) n5 += o.k == 5 && o.ncontrols == 0;
    printf("brickwork n=30 depth 20: %zu gates -> %zu ops, %d of them 5-qubit blocks\n", ops.size(), fo.size(), n5);
  }
  printf("fusion cases 60 worst relative error %.3g failures %d\n", worst, fails);
  return fails ? 1 : 0;
}
