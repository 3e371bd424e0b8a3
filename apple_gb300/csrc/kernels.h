// Host-callable kernel launchers (fem_eval.cu, solver.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "agb_internal.h"

namespace agb {

// bytes of one reduction partial for a precision
inline size_t partial_bytes(int precision) { return precision == AGB_F64 ? 8 : 8; }
inline size_t real_bytes(int precision) { return precision == AGB_F64 ? 8 : 4; }
inline size_t v4_bytes(int precision) { return 4 * real_bytes(precision); }

// u_int[i] = (u_user[3 k], u_user[3 k + 1], u_user[3 k + 2], w) with
// k = user_of_internal[i]; same for p when non-null.
cudaError_t launch_pack(int precision, int n_points, const int32_t* user_of_internal,
                        const void* u_user, void* u_int, const void* p_user, void* p_int,
                        cudaStream_t stream);

// Fused element pass over all tiles of `fv` (AGB_* flags).  Vector results
// go to slots[q * n_slots + slot_of_tv[tv]] for q = 0 grad, 1 diag, 2 prod;
// scalar results are ADDED to *energy / *quad by the last block.
cudaError_t launch_fem_eval(int precision, const FemView& fv, unsigned flags, const void* u_int,
                            const void* p_int, const int32_t* slot_of_tv, void* slots,
                            int32_t n_slots, void* partials, unsigned* counter, double* energy,
                            double* quad, cudaStream_t stream);

// Sum slots per vertex (CSR `off`) and ADD to the caller's (n_points, 3)
// arrays; with `force` (V4, device order) add -f to grad and -f.u to *energy.
cudaError_t launch_unpack(int precision, int n_points, const int32_t* user_of_internal,
                          const int32_t* off, const void* slots, int32_t n_slots, unsigned flags,
                          void* grad, void* diag, void* prod, const void* force, const void* u_int,
                          void* partials, unsigned* counter, double* energy, cudaStream_t stream);

int unpack_blocks(int n_points);

// free/fixed DOF maps: free[i] = full[free_idx[i]];
// full[j] = slot[j] >= 0 ? free[slot[j]] : (fill ? fill[j] : 0)
cudaError_t launch_dof_to_free(int precision, int64_t n_free, const int64_t* free_idx, const void* full,
                               void* free_out, cudaStream_t stream);
cudaError_t launch_dof_to_full(int precision, int64_t n_full, const int32_t* slot, const void* free_in,
                               const void* fill, void* full_out, cudaStream_t stream);

}  // namespace agb
