// Engine-side gate fusion into blocks of at most 5 qubits (host code).
//
// The reference fuses at the circuit level (Circuit.fuse, models/circuit.py:
// 954-1003, producing FusedGate blocks, gates/special.py:28-153, whose matrix
// is Backend.matrix_fused, backends/abstract.py:2680-2717).  qgb_apply_circuit
// with QGB_PLAN_FUSE fuses the gate list itself, so that every caller's
// circuit reaches the tensor-core block kernels, whatever fusion (if any) its
// front end did.
//
// Greedy forward scan.  Each gate acts on a qubit set Q (targets and
// controls).  It joins the most recently created block that touches Q if the
// union stays within 5 qubits; a gate that touches no block commutes with all
// of them and joins the latest block with room; otherwise it opens a new
// block.  A gate on more than 5 qubits becomes a closed block of its own.
// Blocks are emitted in creation order: a gate only ever joins a block
// created at or after the blocks of the earlier gates it shares qubits with,
// and no later block touches the qubits of the gate it just took, so the
// order of non-commuting gates is kept.  A block holding a single gate is
// emitted as that gate (the classifier keeps its cheap kernels); others as
// one dense, uncontrolled op with its 2^q x 2^q matrix, qubits in the order
// they joined (first = most significant matrix bit).  With pad_nqubits set,
// every block (lone gates too) is widened to 5 qubits with the identity on
// the lowest-numbered qubits it lacks: all of them then run on the tensor
// cores, one pass each, and runs of them are not broken by small blocks.
#include <algorithm>
#include <complex>
#include <vector>

#include "qgb_plan.h"

namespace {

typedef std::complex<double> cd;

struct Block {
  std::vector<int> qubits;  // block qubit order: qubits[0] is the most significant matrix bit
  std::vector<cd> U;        // 2^q x 2^q, row-major
  std::vector<int> ops;     // original op indices
  bool closed = false;
};

bool touches(const Block& b, const std::vector<int>& q) {
  for (int x : q)
    if (std::find(b.qubits.begin(), b.qubits.end(), x) != b.qubits.end()) return true;
  return false;
}

int union_size(const Block& b, const std::vector<int>& q) {
  int u = (int)b.qubits.size();
  for (int x : q)
    if (std::find(b.qubits.begin(), b.qubits.end(), x) == b.qubits.end()) ++u;
  return u;
}

// Append qubit x as the new least significant block bit: U <- U (x) I2.
void add_qubit(Block& b, int x) {
  const int d = 1 << b.qubits.size();
  std::vector<cd> V((size_t)4 * d * d, cd(0, 0));
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      const cd u = b.U[(size_t)r * d + c];
      V[(size_t)(2 * r) * (2 * d) + 2 * c] = u;
      V[(size_t)(2 * r + 1) * (2 * d) + 2 * c + 1] = u;
    }
  b.U.swap(V);
  b.qubits.push_back(x);
}

// U <- G U with G the op (controls all 1, targets in matrix order) embedded
// in the block's qubit order: G applied to every column of U, one group of
// 2^k rows (the targets' bits over a base with the controls set) at a time.
void apply_op(Block& b, const qgb_op& op, const double* m) {
  const int q = (int)b.qubits.size(), d = 1 << q, k = op.k, dk = 1 << k;
  auto bit_of = [&](int qubit) {
    const int p = (int)(std::find(b.qubits.begin(), b.qubits.end(), qubit) - b.qubits.begin());
    return q - 1 - p;  // index bit of that qubit within the block
  };
  int tbit[5], cmask = 0, tmask = 0;
  for (int j = 0; j < k; ++j) {
    tbit[j] = bit_of(op.qubits[j]);
    tmask |= 1 << tbit[j];
  }
  for (int j = 0; j < op.ncontrols; ++j) cmask |= 1 << bit_of(op.controls[j]);
  int offs[32];  // row offset of target pattern a (matrix order)
  for (int a = 0; a < dk; ++a) {
    offs[a] = 0;
    for (int j = 0; j < k; ++j)
      if ((a >> (k - 1 - j)) & 1) offs[a] |= 1 << tbit[j];
  }
  double* U = reinterpret_cast<double*>(b.U.data());  // (re, im) pairs, row-major
  bool diag = true;
  for (int r = 0; r < dk && diag; ++r)
    for (int a = 0; a < dk; ++a)
      if (a != r && (m[2 * (r * dk + a)] != 0.0 || m[2 * (r * dk + a) + 1] != 0.0)) {
        diag = false;
        break;
      }
  if (diag) {  // diagonal gates (CZ, phases): scale the rows whose entry is not 1
    for (int a = 0; a < dk; ++a) {
      const double gr = m[2 * (a * dk + a)], gi = m[2 * (a * dk + a) + 1];
      if (gr == 1.0 && gi == 0.0) continue;
      for (int base = 0; base < d; ++base) {
        if ((base & tmask) || (base & cmask) != cmask) continue;
        double* u = U + 2 * (size_t)(base | offs[a]) * d;
        for (int c = 0; c < 2 * d; c += 2) {
          const double xr = u[c], xi = u[c + 1];
          u[c] = gr * xr - gi * xi;
          u[c + 1] = gr * xi + gi * xr;
        }
      }
    }
    return;
  }
  if (dk == 2) {  // dense 1-qubit gates: an operation on two whole rows per group
    const double g00r = m[0], g00i = m[1], g01r = m[2], g01i = m[3];
    const double g10r = m[4], g10i = m[5], g11r = m[6], g11i = m[7];
    for (int base = 0; base < d; ++base) {
      if ((base & tmask) || (base & cmask) != cmask) continue;
      double* u0 = U + 2 * (size_t)(base | offs[0]) * d;
      double* u1 = U + 2 * (size_t)(base | offs[1]) * d;
      for (int c = 0; c < 2 * d; c += 2) {
        const double x0r = u0[c], x0i = u0[c + 1], x1r = u1[c], x1i = u1[c + 1];
        u0[c] = (g00r * x0r - g00i * x0i) + (g01r * x1r - g01i * x1i);
        u0[c + 1] = (g00r * x0i + g00i * x0r) + (g01r * x1i + g01i * x1r);
        u1[c] = (g10r * x0r - g10i * x0i) + (g11r * x1r - g11i * x1i);
        u1[c + 1] = (g10r * x0i + g10i * x0r) + (g11r * x1i + g11i * x1r);
      }
    }
    return;
  }
  double inr[32], ini[32];
  for (int base = 0; base < d; ++base) {
    if ((base & tmask) || (base & cmask) != cmask) continue;  // group representative, controls set
    for (int c = 0; c < d; ++c) {
      for (int a = 0; a < dk; ++a) {
        const double* u = U + 2 * ((size_t)(base | offs[a]) * d + c);
        inr[a] = u[0];
        ini[a] = u[1];
      }
      for (int r = 0; r < dk; ++r) {
        double ar = 0.0, ai = 0.0;
        const double* g = m + 2 * r * dk;
        for (int a = 0; a < dk; ++a) {
          ar += g[2 * a] * inr[a] - g[2 * a + 1] * ini[a];
          ai += g[2 * a] * ini[a] + g[2 * a + 1] * inr[a];
        }
        double* u = U + 2 * ((size_t)(base | offs[r]) * d + c);
        u[0] = ar;
        u[1] = ai;
      }
    }
  }
}

}  // namespace

// The fused gate list of ops[0..nops): records in *ops_out, their matrices in
// *coefs_out (coef_offset into it).  Host work: every gate is applied once to
// its block's 2^q x 2^q matrix (at most 32 x 32 x 2^k multiply-adds).
void qgb_fuse5(const qgb_op* ops, int nops, const double* coefs, std::vector<qgb_op>* ops_out,
               std::vector<double>* coefs_out, int pad_nqubits) {
  std::vector<Block> blocks;
  for (int i = 0; i < nops; ++i) {
    const qgb_op& op = ops[i];
    std::vector<int> Q(op.qubits, op.qubits + op.k);
    Q.insert(Q.end(), op.controls, op.controls + op.ncontrols);
    int target = -1;
    if ((int)Q.size() <= 5) {
      int latest = -1;  // the most recent block touching Q
      for (int b = (int)blocks.size() - 1; b >= 0; --b)
        if (touches(blocks[b], Q)) {
          latest = b;
          break;
        }
      if (latest >= 0) {
        if (!blocks[latest].closed && union_size(blocks[latest], Q) <= 5) target = latest;
      } else {
        for (int b = (int)blocks.size() - 1; b >= 0; --b)  // commutes with every block so far
          if (!blocks[b].closed && union_size(blocks[b], Q) <= 5) {
            target = b;
            break;
          }
      }
    }
    if (target < 0) {
      blocks.emplace_back();
      blocks.back().U.assign(1, cd(1, 0));
      blocks.back().closed = (int)Q.size() > 5;
      target = (int)blocks.size() - 1;
    }
    Block& b = blocks[target];
    b.ops.push_back(i);
    if (b.closed) {
      b.qubits = Q;  // no matrix, but later gates on these qubits must stay after it
    } else {
      for (int x : Q)
        if (std::find(b.qubits.begin(), b.qubits.end(), x) == b.qubits.end()) add_qubit(b, x);
      apply_op(b, op, coefs + op.coef_offset);
    }
  }
  ops_out->clear();
  coefs_out->clear();
  for (Block& b : blocks) {
    if (pad_nqubits >= 5 && !b.closed)  // identity on extra qubits: every block a 5-qubit block
      for (int x = 0; x < pad_nqubits && (int)b.qubits.size() < 5; ++x)
        if (std::find(b.qubits.begin(), b.qubits.end(), x) == b.qubits.end()) add_qubit(b, x);
    if (b.closed || (b.ops.size() == 1 && (int)b.qubits.size() < 5)) {  // a lone gate keeps its own op and matrix
      qgb_op o = ops[b.ops[0]];
      const int m = 2 << (2 * o.k);
      o.coef_offset = (int64_t)coefs_out->size();
      coefs_out->insert(coefs_out->end(), coefs + ops[b.ops[0]].coef_offset, coefs + ops[b.ops[0]].coef_offset + m);
      ops_out->push_back(o);
      continue;
    }
    qgb_op o = qgb_op();
    o.k = (int32_t)b.qubits.size();
    o.ncontrols = 0;
    for (int j = 0; j < o.k; ++j) o.qubits[j] = b.qubits[j];
    o.coef_offset = (int64_t)coefs_out->size();
    for (const cd& u : b.U) {
      coefs_out->push_back(u.real());
      coefs_out->push_back(u.imag());
    }
    ops_out->push_back(o);
  }
}

extern "C" int qgb_fuse_stats(const qgb_op* ops, int nops, const double* coefs, int pad_nqubits, int* nops_out,
                              int* nblocks5) {
  if (nops < 0 || (nops > 0 && (!ops || !coefs)) || !nops_out || !nblocks5) {
    qgb_set_error("qgb_fuse_stats: bad arguments");
    return QGB_ERR_INVALID;
  }
  std::vector<qgb_op> fo;
  std::vector<double> fc;
  qgb_fuse5(ops, nops, coefs, &fo, &fc, pad_nqubits >= 5 ? pad_nqubits : 0);
  *nops_out = (int)fo.size();
  *nblocks5 = 0;
  for (const qgb_op& o : fo) *nblocks5 += o.k == 5 && o.ncontrols == 0;
  return QGB_OK;
}
