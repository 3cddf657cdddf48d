// Host-side check of the complex128 tensor-core block kernel (Ozaki scheme).
//
// Includes qgb_tc128.cu and replays k_fused5_oz on the CPU with the tables
// make_oz_geom builds and the same digit / combine functions the kernel
// calls: tile scale, balanced digits into the bf16 A slices (decoded back
// from their byte offsets), the stacked B slices, the level accumulators as
// exact integer sums (checked below 2^24, hence exact in FP32), the
// combination into doubles and the stores (row and column offsets).  Compares with
// the block applied in FP64 for n = 12..15 and random, lowest and highest
// block placements, plus states with a wide dynamic range: every output must
// be within 2^-41 of 2^(E + F) (E, F the exponents of its tile and gate-row
// scales, the worst-case bound of the fixed-point rounding over K = 64), and
// the largest error over a Gaussian state within 1e-13 of its largest output.
// Also counts shared-memory wavefronts of the A writes (4-byte).  Then replays chains of three unitary
// blocks in the fixed-point state format (k_fused5_oz<true> between
// oz_to_fix and oz_from_fix) against the FP64 product.
// No kernel is launched.
#include <complex>
#include <cstdio>
#include <map>
#include <random>
#include <set>

#include "qgb_tc128.cu"

typedef std::complex<double> cd;

static i64 host_tile_base(i64 t, const OzGeom& geo) {
  i64 base = 0;
  for (int b = 0; b < geo.nrest; ++b) base |= ((t >> b) & 1) << geo.rest[b];
  return base;
}

// wavefronts of one warp access: `width` bytes per lane at byte offsets off[32]
static int wavefronts(const uint32_t* off, int width) {
  const int group = 128 / width;  // lanes served per wavefront without conflicts
  int total = 0;
  for (int g0 = 0; g0 < 32; g0 += group) {
    std::map<int, std::set<uint32_t>> bank;
    for (int l = g0; l < g0 + group; ++l)
      for (int w = 0; w < width / 4; ++w) bank[(off[l] / 4 + w) % 32].insert(off[l] / 4 + w);
    int m = 0;
    for (auto& kv : bank) m = std::max<int>(m, (int)kv.second.size());
    total += m;
  }
  return total;
}

// One launch of k_fused5_oz<true> replayed on a fixed-point state (X holds
// the re, im integers of each amplitude): one shift for the launch from the
// OR of the state's high words' magnitudes, byte digits (oz_fix_z,
// oz_zdigits), exact level sums, oz_combine_fix, direct stores.
static void replay_fix_block(std::vector<int64_t>& X, int n, const GateOp& g, int* exact_fails) {
  OzGeom* geo = new OzGeom();
  OzGate* G = new OzGate();
  int cbit[5];
  make_oz_geom(n, g.tbits, geo, cbit);
  make_oz_gate(g, cbit, G, true);
  static int Bd[OZ_NSLICE][64][64];
  for (int nn = 0; nn < 64; ++nn)
    for (int k = 0; k < 64; ++k) {
      const int r = nn >> 1, c = k >> 1;
      const double v = (nn & 1) == 0 ? ((k & 1) == 0 ? G->ur[r][c] : -G->ui[r][c])
                                     : ((k & 1) == 0 ? G->ui[r][c] : G->ur[r][c]);
      int d[OZ_NSLICE];
      oz_digits(v, G->fexp[r], d);
      for (int j = 0; j < OZ_NSLICE; ++j) Bd[j][nn][k] = d[j];
    }
  std::map<uint32_t, std::pair<int, int>> dec;
  for (int row = 0; row < 128; ++row)
    for (int c = 0; c < 32; ++c)
      dec[(c >> 2) * geo->a_lbo + (row >> 3) * OZ_A_SBO + (row & 7) * 16 + (c & 3) * 4] = {row, c};
  // the launch's shift: top bit of the OR of |high word| over the state
  // (written by the previous launch or the conversion), as the kernel reads it
  uint32_t o = 0;
  uint64_t exact = 0;
  for (size_t i = 0; i < X.size(); ++i) {
    o |= (uint32_t)std::abs((int32_t)((uint64_t)X[i] >> 32));
    exact |= (uint64_t)(X[i] < 0 ? -X[i] : X[i]);
  }
  const int ph = o ? 31 - __builtin_clz(o) : -1;
  const int sh = ph > 14 ? ph - 14 : 0;
  // the shift keeps every value within 47 bits, and is at most one above
  // the exact one
  {
    const int p = exact ? 63 - oz_clz64(exact) : -1;
    if ((exact >> sh) >= (1ull << 47) || sh > (p > 46 ? p - 46 : 0) + 1) (*exact_fails)++;
  }
  const int64_t bias = oz_fix_bias(sh);
  const i64 ntiles = (i64)1 << (n - 12);
  std::vector<int64_t> Xout(X.size());
  for (i64 t = 0; t < ntiles; ++t) {
    const i64 base = host_tile_base(t, *geo);
    auto gidx = [&](int tid, int r) {
      return base + (tid & 127) + ((tid >> 7) ? geo->g7 : 0) + geo->ghi[r];
    };
    static int Ad[OZ_NSLICE][128][64];
    for (int r = 0; r < OZ_STEPS; ++r)
      for (int tid = 0; tid < OZ_GROUP; ++tid) {
        const auto rc = dec[geo->aoff_lo[tid] + geo->aoff_hi[r]];
        const i64 gi = gidx(tid, r);
        float fre[OZ_NSLICE], fim[OZ_NSLICE];
        oz_zdigits(oz_fix_z(X[2 * gi], sh, bias), fre);
        oz_zdigits(oz_fix_z(X[2 * gi + 1], sh, bias), fim);
        int dre[OZ_NSLICE], dim[OZ_NSLICE];
        for (int s = 0; s < OZ_NSLICE; ++s) {
          dre[s] = (int)fre[s];
          dim[s] = (int)fim[s];
          if ((float)dre[s] != fre[s] || (float)dim[s] != fim[s]) (*exact_fails)++;
        }
        for (int s = 0; s < OZ_NSLICE; ++s) {
          if (std::abs(dre[s]) > 128 || std::abs(dim[s]) > 128) (*exact_fails)++;
          Ad[s][rc.first][2 * rc.second] = dre[s];
          Ad[s][rc.first][2 * rc.second + 1] = dim[s];
        }
      }
    for (int row = 0; row < 128; ++row)
      for (int c = 0; c < 32; ++c)
        for (int part = 0; part < 2; ++part) {
          float acc[OZ_NLEVEL];
          for (int l = 0; l < OZ_NLEVEL; ++l) {
            int64_t sum = 0;
            for (int i = std::max(0, l - (OZ_NSLICE - 1)); i <= std::min(l, OZ_NSLICE - 1); ++i)
              for (int k = 0; k < 64; ++k) sum += (int64_t)Ad[i][row][k] * Bd[l - i][2 * c + part][k];
            if (std::llabs(sum) >= (1ll << 24)) (*exact_fails)++;
            acc[l] = (float)sum;
          }
          // the epilogue's direct store of (row, c)
          Xout[2 * (base + geo->rowoff[row] + geo->coloff[c]) + part] =
              oz_combine_fix(acc, oz_shift(sh + G->fexp[0] - 1029));
        }
  }
  X = Xout;
  delete geo;
  delete G;
}

// A chain of three random unitary blocks in the fixed-point format (scale
// from the FP64 norm, oz_to_fix / oz_from_fix at the ends) against the FP64
// product: 1e-13 absolute on normalised states, including one whose
// amplitudes span 2^-30..1.  Returns the number of failures.
// Trials 4-7 scale the columns of each unitary by factors in [0.5, 1.5]:
// non-unitary blocks (the density-matrix channels' case), chained with the
// headroom of their growth bits (qgb_oz_growth_bits) added to the scale.
static int chain_check(std::mt19937_64& rng, int* exact_fails) {
  std::normal_distribution<double> nd;
  std::uniform_real_distribution<double> ud(0.5, 1.5);
  int fails = 0;
  for (int trial = 0; trial < 8; ++trial) {
    const bool grow = trial >= 4;
    const int n = 13 + (trial & 1);
    const i64 N = (i64)1 << n;
    std::vector<cd> psi(N);
    double nrm2 = 0;
    for (auto& x : psi) {
      x = cd(nd(rng), nd(rng));
      if (trial >= 2) x *= std::ldexp(1.0, -(int)(rng() % 30));
      nrm2 += std::norm(x);
    }
    for (auto& x : psi) x /= std::sqrt(nrm2);
    nrm2 = 0;
    for (auto& x : psi) nrm2 += std::norm(x);
    // the three blocks first (their growth sets the chain's headroom)
    std::vector<GateOp> gs(3);
    std::vector<std::vector<cd>> Us(3);
    int head = 0;
    for (int b = 0; b < 3; ++b) {
      std::vector<int> all(n);
      for (int i = 0; i < n; ++i) all[i] = i;
      std::shuffle(all.begin(), all.end(), rng);
      GateOp g;
      g.kind = GK_DENSE;
      g.tbits.assign(all.begin(), all.begin() + 5);
      // a random unitary: Gram-Schmidt on a complex Gaussian matrix (columns)
      std::vector<cd> U(1024);
      for (auto& u : U) u = cd(nd(rng), nd(rng));
      for (int j = 0; j < 32; ++j) {
        for (int k = 0; k < j; ++k) {
          cd dot = 0;
          for (int i = 0; i < 32; ++i) dot += std::conj(U[i * 32 + k]) * U[i * 32 + j];
          for (int i = 0; i < 32; ++i) U[i * 32 + j] -= dot * U[i * 32 + k];
        }
        double nn = 0;
        for (int i = 0; i < 32; ++i) nn += std::norm(U[i * 32 + j]);
        for (int i = 0; i < 32; ++i) U[i * 32 + j] /= std::sqrt(nn);
      }
      if (grow)
        for (int j = 0; j < 32; ++j) {
          const double f = ud(rng);
          for (int i = 0; i < 32; ++i) U[i * 32 + j] *= f;
        }
      g.coef.resize(1024);
      for (int i = 0; i < 1024; ++i) g.coef[i] = zd(U[i].real(), U[i].imag());
      if (qgb_oz_unitary(g) == grow) fails++;
      const int gb = qgb_oz_growth_bits(g);
      if (grow ? gb != 1 : gb != 0) fails++;  // singular values in [0.5, 1.5]: one bit
      head += gb;
      gs[b] = g;
      Us[b] = U;
    }
    const int e = oz_scale_exp(nrm2) + head;
    std::vector<int64_t> X(2 * N);
    for (i64 i = 0; i < N; ++i) {
      X[2 * i] = oz_to_fix(psi[i].real(), e);
      X[2 * i + 1] = oz_to_fix(psi[i].imag(), e);
    }
    std::vector<cd> ref = psi;
    for (int b = 0; b < 3; ++b) {
      const GateOp& g = gs[b];
      const std::vector<cd>& U = Us[b];
      replay_fix_block(X, n, g, exact_fails);
      std::vector<cd> out(N);
      for (i64 i = 0; i < N; ++i) {
        int bi = 0;
        for (int jt = 0; jt < 5; ++jt) bi |= (int)((i >> g.tbits[jt]) & 1) << (4 - jt);
        if (bi) continue;
        i64 id[32];
        for (int q = 0; q < 32; ++q) {
          id[q] = i;
          for (int jt = 0; jt < 5; ++jt)
            if ((q >> (4 - jt)) & 1) id[q] |= (i64)1 << g.tbits[jt];
        }
        for (int r = 0; r < 32; ++r) {
          cd acc = 0;
          for (int c = 0; c < 32; ++c) acc += U[r * 32 + c] * ref[id[c]];
          out[id[r]] = acc;
        }
      }
      ref = out;
    }
    double err = 0, big = 0;
    for (i64 i = 0; i < N; ++i) {
      err = std::max(err, std::abs(cd(oz_from_fix(X[2 * i], e), oz_from_fix(X[2 * i + 1], e)) - ref[i]));
      big = std::max(big, std::abs(ref[i]));
      // the fixed-point range holds: |X| < 2^61 after every block
      if (std::llabs(X[2 * i]) >= (1ll << 61) || std::llabs(X[2 * i + 1]) >= (1ll << 61)) (*exact_fails)++;
    }
    printf("fixed-point chain n=%d trial %d (headroom %d): max abs error %.3g\n", n, trial, head, err);
    if (err > 1e-13 * std::max(1.0, std::ldexp(1.0, head))) fails++;
  }
  return fails;
}

int main() {
  std::mt19937_64 rng(11);
  std::normal_distribution<double> nd;
  int fails = 0, cases = 0, bank_fails = 0, exact_fails = 0;
  double worst = 0;
  for (int n = 12; n <= 15; ++n) {
    for (int trial = 0; trial < 16; ++trial) {
      std::vector<int> all(n);
      for (int i = 0; i < n; ++i) all[i] = i;
      std::shuffle(all.begin(), all.end(), rng);
      std::vector<int> tb(all.begin(), all.begin() + 5);
      if (trial == 0) tb = {4, 3, 2, 1, 0};
      if (trial == 1) tb = {n - 1, n - 2, n - 3, n - 4, n - 5};
      if (trial == 2) tb = {2, 0, 1, 9, 3};
      GateOp g;
      g.kind = GK_DENSE;
      g.tbits = tb;
      g.coef.resize(1024);
      for (auto& c : g.coef) c = zd(nd(rng), nd(rng)) * 0.2;
      OzGeom* geo = new OzGeom();
      OzGate* G = new OzGate();
      int cbit[5];
      make_oz_geom(n, tb, geo, cbit);
      make_oz_gate(g, cbit, G, false);
      // paired stores exactly when index bit 0 is a block qubit
      if (geo->pair != (int)(std::find(tb.begin(), tb.end(), 0) != tb.end())) fails++;
      int t5 = 0;
      for (int b : tb) t5 += b < 5;
      const i64 N = (i64)1 << n;
      std::vector<cd> psi(N), out(N, cd(0, 0)), ref(N);
      std::vector<double> bound(N, 0.0);
      const bool wide = trial % 4 == 3;  // amplitudes over ~2^-40 .. 1
      for (auto& x : psi) {
        x = cd(nd(rng), nd(rng));
        if (wide) x *= std::ldexp(1.0, -(int)(rng() % 40));
      }
      for (i64 i = 0; i < N; ++i) {  // the block applied directly
        int bi = 0;
        for (int jt = 0; jt < 5; ++jt) bi |= (int)((i >> tb[jt]) & 1) << (4 - jt);
        if (bi) continue;
        i64 id[32];
        for (int b = 0; b < 32; ++b) {
          id[b] = i;
          for (int jt = 0; jt < 5; ++jt)
            if ((b >> (4 - jt)) & 1) id[b] |= (i64)1 << tb[jt];
        }
        for (int r = 0; r < 32; ++r) {
          cd acc = 0;
          for (int c = 0; c < 32; ++c) acc += cd(g.coef[r * 32 + c].real(), g.coef[r * 32 + c].imag()) * psi[id[c]];
          ref[id[r]] = acc;
        }
      }
      // stacked B slices as integers: Bd[j][n][k]
      static int Bd[OZ_NSLICE][64][64];
      for (int nn = 0; nn < 64; ++nn)
        for (int k = 0; k < 64; ++k) {
          const int r = nn >> 1, c = k >> 1;
          double v;
          if ((nn & 1) == 0) v = (k & 1) == 0 ? G->ur[r][c] : -G->ui[r][c];
          else v = (k & 1) == 0 ? G->ui[r][c] : G->ur[r][c];
          int d[OZ_NSLICE];
          oz_digits(v, G->fexp[r], d);
          for (int j = 0; j < OZ_NSLICE; ++j) {
            Bd[j][nn][k] = d[j];
            if (oz_boff(192 * (nn >> 5) + 32 * j + (nn & 31), k) + 2 > 8 * OZ_B_LBO) exact_fails++;
          }
        }
      std::map<uint32_t, std::pair<int, int>> dec;  // A slice byte offset of (row, c) pair
      for (int row = 0; row < 128; ++row)
        for (int c = 0; c < 32; ++c)
          dec[(c >> 2) * geo->a_lbo + (row >> 3) * OZ_A_SBO + (row & 7) * 16 + (c & 3) * 4] = {row, c};
      std::vector<int> seen(N, 0), wrote(N, 0);
      bool bad = false;
      const i64 ntiles = (i64)1 << (n - 12);
      for (i64 t = 0; t < ntiles; ++t) {
        const i64 base = host_tile_base(t, *geo);
        int exm = 0;
        for (int r = 0; r < OZ_STEPS; ++r)
          for (int tid = 0; tid < OZ_GROUP; ++tid) {
            const i64 gi = base + (tid & 127) + ((tid >> 7) ? geo->g7 : 0) + geo->ghi[r];
            if (gi < 0 || gi >= N) { bad = true; continue; }
            exm = std::max(exm, (int)((oz_dbits(psi[gi].real()) >> 52) & 0x7FF));
            exm = std::max(exm, (int)((oz_dbits(psi[gi].imag()) >> 52) & 0x7FF));
          }
        static int Ad[OZ_NSLICE][128][64];
        std::set<uint32_t> used;
        for (int r = 0; r < OZ_STEPS; ++r) {
          for (int tid = 0; tid < OZ_GROUP; ++tid) {
            const i64 gi = base + (tid & 127) + ((tid >> 7) ? geo->g7 : 0) + geo->ghi[r];
            if (gi < 0 || gi >= N) { bad = true; continue; }
            seen[gi]++;
            const uint32_t o = geo->aoff_lo[tid] + geo->aoff_hi[r];
            if (o + 4 > (uint32_t)OZ_A_SLICE || !dec.count(o) || used.count(o)) { bad = true; continue; }
            used.insert(o);
            const auto rc = dec[o];
            int dre[OZ_NSLICE], dim[OZ_NSLICE];
            oz_digits(psi[gi].real(), exm, dre);
            oz_digits(psi[gi].imag(), exm, dim);
            for (int s = 0; s < OZ_NSLICE; ++s) {
              // the packed bf16 pair decodes to the digits
              const uint32_t w = oz_pack((float)dre[s], (float)dim[s]);
              uint32_t lo = (w & 0xFFFF) << 16, hi = w & 0xFFFF0000u;
              float flo, fhi;
              memcpy(&flo, &lo, 4);
              memcpy(&fhi, &hi, 4);
              if (flo != (float)dre[s] || fhi != (float)dim[s] || std::abs(dre[s]) > 128 || std::abs(dim[s]) > 128)
                exact_fails++;
              Ad[s][rc.first][2 * rc.second] = dre[s];
              Ad[s][rc.first][2 * rc.second + 1] = dim[s];
            }
          }
          if (t == 0)
            for (int w = 0; w < OZ_GROUP / 32; ++w) {
              uint32_t off[32];
              for (int l = 0; l < 32; ++l) off[l] = geo->aoff_lo[32 * w + l] + geo->aoff_hi[r];
              if (wavefronts(off, 4) > (t5 >= 2 ? 1 : t5 == 1 ? 2 : 4)) bank_fails++;
            }
        }
        for (int row = 0; row < 128; ++row)
          for (int c = 0; c < 32; ++c) {
            double vals[2];
            for (int part = 0; part < 2; ++part) {
              const int nn = 2 * c + part;
              float acc[OZ_NLEVEL];
              for (int l = 0; l < OZ_NLEVEL; ++l) {
                int64_t sum = 0;
                for (int i = std::max(0, l - (OZ_NSLICE - 1)); i <= std::min(l, OZ_NSLICE - 1); ++i)
                  for (int k = 0; k < 64; ++k) sum += (int64_t)Ad[i][row][k] * Bd[l - i][nn][k];
                if (std::llabs(sum) >= (1ll << 24)) exact_fails++;
                acc[l] = (float)sum;
              }
              vals[part] = oz_combine(acc, exm + G->fexp[c] - 2098);
            }
            // the epilogue's direct store of (row, c); with geo->pair, outputs
            // c and c + 1 (c even) go out as one 32-byte store at gi
            const i64 gi = base + geo->rowoff[row] + geo->coloff[c];
            if (gi < 0 || gi >= N) { bad = true; continue; }
            if (geo->pair && (c & 1) == 0 && ((gi & 1) || base + geo->rowoff[row] + geo->coloff[c + 1] != gi + 1))
              bad = true;
            wrote[gi]++;
            out[gi] = cd(vals[0], vals[1]);
            bound[gi] = std::ldexp(1.0, (exm - 1022) + (G->fexp[c] - 1022) - 41);
          }
      }
      double err = 0, nrm = 0;
      int over = 0;
      for (i64 i = 0; i < N; ++i) {
        if (seen[i] != 1 || wrote[i] != 1) bad = true;
        const double e = std::max(std::abs(out[i].real() - ref[i].real()), std::abs(out[i].imag() - ref[i].imag()));
        if (e > bound[i]) over++;
        err = std::max(err, std::abs(out[i] - ref[i]));
        nrm = std::max(nrm, std::abs(ref[i]));
      }
      ++cases;
      if (!wide) worst = std::max(worst, err / nrm);
      if (bad || over || (!wide && err > 1e-13 * nrm)) {
        ++fails;
        printf("FAIL n=%d block bits %d,%d,%d,%d,%d rel err=%g bad=%d\n", n, tb[0], tb[1], tb[2], tb[3], tb[4],
               err / nrm, (int)bad);
        printf("  outputs over the bound: %d\n", over);
      }
      delete geo;
      delete G;
    }
  }
  printf("cases %d worst relative error (Gaussian states) %.3g\n", cases, worst);
  fails += chain_check(rng, &exact_fails);
  printf("index failures %d exactness failures %d bank-pattern failures %d\n", fails, exact_fails, bank_fails);
  return (fails || exact_fails || bank_fails) ? 1 : 0;
}
