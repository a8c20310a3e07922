// Random 32 B sector probe: the L2 and HBM ceilings of the transport kernel's access pattern.
//
// Every voxel-ID fetch and every tally update of the transport is a data-dependent,
// uncoalesced access to one 32 B sector (the unit the L2 and the DRAM controllers move).  The
// copy bandwidth of a streaming kernel overstates what such accesses can reach, so this probe
// issues the same kind of traffic with as many requests in flight as the SMs allow: each
// thread touches `iters` sectors chosen by a 32-bit integer hash of its request index, either
// loading 4 bytes cached in L2 only (ld.global.cg: no L1 reuse, as for a voxel fetch of a
// photon that moved) or adding 1 to a 64-bit word (a RED, as for a tally record).  Footprints
// that fit the L2 give the L2 ceiling, larger ones the HBM ceiling.
//
// Every address is `sector & mask` of a buffer of mask + 1 sectors (a power of two checked on
// the host), so no access leaves the buffer.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/midsx_gpu.h"
#include "tables_internal.h"

namespace {

constexpr int kProbeBlock = 256;
constexpr int kProbeUnroll = 8;

// A bijective 32-bit mix (multiply-xorshift): consecutive request indexes land on unrelated
// sectors, and distinct indexes on distinct hashes.
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x *= 0x9E3779B1u;
    x ^= x >> 15;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    return x;
}

template <int MODE>
__global__ void __launch_bounds__(kProbeBlock) sector_probe_kernel(uint32_t* __restrict__ buf, uint32_t sector_mask,
                                                                   uint32_t iters, uint32_t seed) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t base = t * iters + seed;
    uint32_t acc = 0;
    for (uint32_t i = 0; i < iters; i += kProbeUnroll) {
        uint32_t s[kProbeUnroll];
#pragma unroll
        for (int j = 0; j < kProbeUnroll; ++j) s[j] = mix32(base + i + j) & sector_mask;
#pragma unroll
        for (int j = 0; j < kProbeUnroll; ++j) {
            if constexpr (MODE == 0) {
                acc += __ldcg(buf + 8ull * s[j]);
            } else {
                atomicAdd(reinterpret_cast<unsigned long long*>(buf + 8ull * s[j]), 1ull);
            }
        }
    }
    // keeps the loads; with a buffer of zeros or small counts the sum never reaches this value
    if (MODE == 0 && acc == 0xFFFFFFFFu) buf[8ull * (t & sector_mask) + 4] = acc;
}

}  // namespace

extern "C" midsx_status midsx_gpu_probe_sectors(void* buf, uint64_t bytes, int32_t mode, uint64_t requests,
                                                uint32_t seed, uint64_t* issued, void* stream) {
    if (!buf || !issued || (mode != 0 && mode != 1) || requests == 0 || bytes < 32 || (bytes & (bytes - 1)) ||
        bytes / 32 > (uint64_t(1) << 32) || (reinterpret_cast<uintptr_t>(buf) & 31)) {
        midsx::set_last_error("midsx_gpu_probe_sectors: buffer must be a 32-byte aligned power-of-two size "
                              "of at most 128 GiB, mode 0 or 1, requests > 0");
        return MIDSX_INVALID_ARG;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        midsx::set_last_error(std::string("midsx_gpu_probe_sectors: ") + cudaGetErrorString(e));
        return MIDSX_CUDA_ERROR;
    }
    // 8 blocks of 256 threads fill an SM's 2048 thread slots
    const uint64_t blocks = uint64_t(sms) * (2048 / kProbeBlock);
    const uint64_t threads = blocks * kProbeBlock;
    uint64_t iters = (requests + threads - 1) / threads;
    iters = (iters + kProbeUnroll - 1) / kProbeUnroll * kProbeUnroll;
    if (threads * iters > (uint64_t(1) << 32)) {
        midsx::set_last_error("midsx_gpu_probe_sectors: more than 2^32 requests");
        return MIDSX_INVALID_ARG;
    }
    const uint32_t mask = uint32_t(bytes / 32 - 1);
    auto s = static_cast<cudaStream_t>(stream);
    if (mode == 0)
        sector_probe_kernel<0><<<unsigned(blocks), kProbeBlock, 0, s>>>(static_cast<uint32_t*>(buf), mask,
                                                                        uint32_t(iters), seed);
    else
        sector_probe_kernel<1><<<unsigned(blocks), kProbeBlock, 0, s>>>(static_cast<uint32_t*>(buf), mask,
                                                                        uint32_t(iters), seed);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        midsx::set_last_error(std::string("midsx_gpu_probe_sectors: ") + cudaGetErrorString(e));
        return MIDSX_CUDA_ERROR;
    }
    *issued = threads * iters;
    return MIDSX_OK;
}
