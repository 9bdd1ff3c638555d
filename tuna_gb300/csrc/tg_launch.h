// tg_launch.h — host-side launchers of the counting kernels (defined in
// tg_phase1.cu, tg_phase2.cu, tg_api.cu) shared by the entry points.
#pragma once
#include <cuda_runtime.h>

#include "tg_internal.cuh"

namespace tg {
size_t cut_smem_bytes(int w, uint32_t p1, bool exp);
cudaError_t launch_pack(const uint8_t* seq, uint64_t n, uint32_t* packed, uint32_t* valid, uint64_t n_words,
                        unsigned long long* n_bases, cudaStream_t st);
cudaError_t launch_cut(const CutParams& P, const HashTables* gT, bool exp, cudaStream_t st);
cudaError_t launch_scan(const uint32_t* in, uint64_t n, unsigned long long* out, unsigned long long* sums,
                        unsigned long long* total, cudaStream_t st, int* launches);
cudaError_t launch_bucket(const BucketParams& P, cudaStream_t st);
size_t count_smem_bytes(int W, uint32_t slots);
size_t key_bytes(int W);
cudaError_t launch_count(int W, const Phase2Params& P, uint32_t grid, cudaStream_t st);
cudaError_t launch_fallback(int W, const FallbackParams& F, uint64_t S, const Phase2Params& P, uint32_t grid,
                            cudaStream_t st, int* launches);

// ntHash roll / init tables for minimizer length m (host side).
HashTables make_hash_tables(int m);

__global__ void k_sizes(const unsigned long long* off_r, uint32_t n_buckets, uint32_t C,
                        unsigned long long* out_recs);
}  // namespace tg
