// Host-side gate classification shared by the per-gate dispatcher and the
// shared-memory pass planner.
#pragma once

#include <complex>
#include <vector>

#include "qgb_common.cuh"

typedef std::complex<double> zd;

enum GateKind {
  GK_PHASE = 0,  // amplitudes with all ``cbits`` set get *coef[0]
  GK_DIAG = 1,   // amplitude *= coef[target bits] where all ``cbits`` set
  GK_XLIKE = 2,  // [[0, a], [b, 0]] on tbits[0] where all ``cbits`` set
  GK_SWAP = 3,   // SWAP of tbits[0], tbits[1] where all ``cbits`` set
  GK_DENSE = 4,  // dense 2^k x 2^k on tbits where all ``cbits`` set
};

struct GateOp {
  int kind;
  std::vector<int> tbits;  // target bit positions, most significant matrix bit first
  std::vector<int> cbits;  // control bit positions (all must be 1)
  std::vector<zd> coef;    // PHASE: 1; DIAG: 2^k; XLIKE: 2 (a, b); SWAP: 0; DENSE: 4^k row-major
  bool identity = false;   // a PHASE of exactly 1: nothing to do
};

// Validate a gate and reduce it to its cheapest form: controls hidden in
// the matrix are extracted, then diagonal / X-like / SWAP / dense.
// Returns a QGB status; on success fills ``op``.
int qgb_classify(int nqubits, const int* qubits, int k, const int* controls, int ncontrols,
                 const double* matrix, GateOp* op, const char* fn);

// Tensor-core block kernels (qgb_tc.cu, qgb_tc128.cu): uncontrolled 5-qubit
// dense blocks.  complex64 3xTF32; complex128 Ozaki scheme (n >= 12), on
// IEEE doubles or, inside a chain, on the fixed-point format.
int qgb_launch_fused5_tc(void* state, int n, const GateOp& g, cudaStream_t s);
int qgb_launch_fused5_oz(void* state, int n, const GateOp& g, cudaStream_t s, bool fix,
                         uint32_t* fix_words = nullptr, int b = 0);
bool qgb_oz_unitary(const GateOp& g);
int qgb_oz_growth_bits(const GateOp& g);
int qgb_run_oz_chain(void* state, int n, const std::vector<const GateOp*>& blocks, cudaStream_t s, int headroom);
int qgb_tc_prepare();  // allocate the tensor-core paths' device buffers (idempotent)
int qgb_oz_stream_prepare(cudaStream_t s);  // complex128 chain scratch of stream s (qgb_tc128.cu)
int qgb_oz_stream_release(cudaStream_t s);  // and its release before the stream is destroyed

// Engine-side fusion into blocks of at most 5 qubits (qgb_fuse.cu).
// pad_nqubits >= 5: widen every block to 5 qubits (identity on the lowest
// qubits of the pad_nqubits-qubit state it lacks); 0: no padding.
void qgb_fuse5(const qgb_op* ops, int nops, const double* coefs, std::vector<qgb_op>* ops_out,
               std::vector<double>* coefs_out, int pad_nqubits);
