// Placeholder for the shared-memory multi-gate planner: runs gate by gate.
#include "qgb_common.cuh"

int qgb_run_blocked(void* state, int nqubits, int dtype, const qgb_op* ops, int nops, const double* coefs,
                    cudaStream_t s) {
  for (int i = 0; i < nops; ++i) {
    int st = qgb_apply_gate(state, nqubits, dtype, ops[i].qubits, ops[i].k, ops[i].controls, ops[i].ncontrols,
                            coefs + ops[i].coef_offset, (void*)s);
    if (st) return st;
  }
  return QGB_OK;
}
