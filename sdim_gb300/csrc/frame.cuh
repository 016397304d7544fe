// Pauli-frame sampler: the reference's route for Program.simulate(shots > 1)
// without record_tableau / force_tableau (sdim/program.py:244-265, 45-165).
// Shot 0 is one noiseless tableau shot (any tableau engine); every other
// shot carries a Pauli frame, x and z residues per qudit, through the
// instruction list and records (reference value + x_q) mod d at M / M_X and
// the reference value itself at RESET.  This header is the host-side view:
// the frame instruction format, the descriptor and the launcher (k_frame.cu).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sdim {

// Frame instruction word: x = code | qudit << 8, y = target qudit (codes 9-13)
// or the N1 coin threshold.  Codes 1-16 are the reference's gate ids with
// CZ (11), CZ_INV (12), SWAP (13) and M_X (15) kept whole, because the frame
// rules of the reference act on them directly (sdim/program.py:108-119,
// 128-131); N1 is OP_N1D / OP_N1F / OP_N1P / OP_N1OFF as in the tableau
// stream.  Identity instructions are left out.
constexpr uint32_t FOP_CZ = 11, FOP_CZ_INV = 12, FOP_SWAP = 13, FOP_MX = 15;

// Philox domain of the frame draws: event e of a shot is the initial z of
// qudit e (e < n) or the z drawn after measurement ordinal k (e = n + k);
// word e & 3 of the block with counter ordinal e >> 2 gives the residue.
constexpr uint32_t kDomainFrame = 3;

struct FrameDesc {
  const uint2* ops;    // frame instruction stream
  const uint8_t* ref;  // records of the reference shot (nmeas bytes, device)
  uint8_t* out;        // nshots x nmeas records of the frame shots
  unsigned long long seed;
  long long shot0;     // stream shot index of the first frame shot
  int nops, n, d, nmeas, nshots;
};

// Shared memory of one frame block (one warp of 32 shots).
size_t frame_smem_bytes(int n);
cudaError_t frame_set_smem(int optin);

// One single-warp block per 32 frame shots; false for an unsupported d.
bool launch_frame_pass(int grid, size_t smem, cudaStream_t s, const FrameDesc& fd, int* status);

}  // namespace sdim
