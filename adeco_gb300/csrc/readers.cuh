// readers.cuh -- particle files into a session's resident lattice.
//
// The reference's single-rank readers (src/AdPointDataReaders.h), done on
// the GPU: the file is read on the host in pinned chunks (two buffers, so the
// next chunk is read while the last one is copied and decoded), each chunk is
// decoded by a kernel that writes every particle straight to its lattice site
// (float4, x fastest), and the global bounding box and the periodic unwrap
// run on the device.  Included by runtime.cu (it uses the session's internals).
//
//   SORTED_BY_ID  float32 x, y, z per particle in id order (:770-911); the
//                 reference ignores the stride, and so does this reader.
//   DARK_SKY      SDF: text header up to "# SDF-EOH", sha1_chunks x (4 + 20)
//                 bytes (get_header_size, :425-467), then 32-byte records
//                 {float x, y, z, vx, vy, vz; int64 id} (:508-516).  The id's
//                 low 48 bits are a Morton key, bit 3l -> x, 3l+1 -> y,
//                 3l+2 -> z (morton_2_grid, :366-394); with stride s only
//                 particles on multiples of s are kept, at index / s
//                 (:622-637).
//   unwrap        apply_boundary_corrections (:154-204) over the bbox of the
//                 particles read: per axis, index above n/2 and position
//                 below min + ext/4 -> + ext; index below n/2 and position
//                 above min + (3/4) ext -> - ext; in FP32.
#pragma once

#include <cstdio>
#include <string>

namespace adeco {

constexpr size_t kReadChunk = 32ull << 20;  // bytes per pinned host buffer

__global__ void sorted_chunk_kernel(const float *xyz, long long first, long long count, float4 *lattice)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
        lattice[first + i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f);
}

// every third bit of a 48-bit Morton key, starting at bit 0, packed
__device__ __forceinline__ unsigned long long morton_axis(unsigned long long k)
{
    k &= 0x1249249249249ull;  // bits 0, 3, ..., 45
    k = (k ^ (k >> 2)) & 0x30c30c30c30c3ull;
    k = (k ^ (k >> 4)) & 0xf00f00f00f00full;
    k = (k ^ (k >> 8)) & 0xff0000ff0000ffull;
    k = (k ^ (k >> 16)) & 0xffff00000000ffffull;
    k = (k ^ (k >> 32)) & 0xffffull;
    return k;
}

// DARK_SKY records of a chunk -> lattice sites; kept counts the particles
// placed, error[0] is set for an id outside the lattice
__global__ void darksky_chunk_kernel(const unsigned char *rec, long long count, int n0, int stride, int n,
                                     float4 *lattice, unsigned long long *kept, int *error)
{
    unsigned long long c = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float *f = reinterpret_cast<const float *>(rec + 32 * i);
        const unsigned long long key = *reinterpret_cast<const unsigned long long *>(rec + 32 * i + 24) & ((1ull << 48) - 1);
        const long long lx = (long long)morton_axis(key), ly = (long long)morton_axis(key >> 1),
                        lz = (long long)morton_axis(key >> 2);
        if (lx >= n0 || ly >= n0 || lz >= n0) {
            atomicOr(error, 1);
            continue;
        }
        if (stride != 1 && (lx % stride || ly % stride || lz % stride)) continue;
        const long long id = lx / stride + (long long)n * (ly / stride + (long long)n * (lz / stride));
        lattice[id] = make_float4(f[0], f[1], f[2], 0.f);
        ++c;
    }
    if (c) atomicAdd(kept, c);
}

// periodic unwrap of a whole lattice; lim = {ext, min + ext/4, min + 3/4 ext} per axis
__global__ void unwrap_kernel(float4 *lattice, int n, float half, float3 ext, float3 h1, float3 h2)
{
    const long long total = (long long)n * n * n;
    for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long long)gridDim.x * blockDim.x) {
        float4 p = lattice[id];
        const float ix = (float)(id % n), iy = (float)((id / n) % n), iz = (float)(id / ((long long)n * n));
        if (ix > half && p.x < h1.x) p.x = __fadd_rn(p.x, ext.x);
        else if (ix < half && p.x > h2.x) p.x = __fsub_rn(p.x, ext.x);
        if (iy > half && p.y < h1.y) p.y = __fadd_rn(p.y, ext.y);
        else if (iy < half && p.y > h2.y) p.y = __fsub_rn(p.y, ext.y);
        if (iz > half && p.z < h1.z) p.z = __fadd_rn(p.z, ext.z);
        else if (iz < half && p.z > h2.z) p.z = __fsub_rn(p.z, ext.z);
        lattice[id] = p;
    }
}

struct HostFile {
    std::FILE *f = nullptr;
    ~HostFile()
    {
        if (f) std::fclose(f);
    }
};

// header size of an SDF file by get_header_size's rule
static int sdf_header_size(std::FILE *f, size_t &size)
{
    std::fseek(f, 0, SEEK_SET);
    char line[1024];
    int sha1_chunks = -1;
    for (int c = 0; c < 100000; ++c) {
        if (!std::fgets(line, sizeof line, f)) break;
        const size_t len = std::strlen(line);
        if (len == sizeof line - 1 && line[len - 1] != '\n') break;  // a line the reference cannot read either
        if (std::strncmp(line, "int sha1_chunks =", 17) == 0) sha1_chunks = std::atoi(line + 17);
        if (std::strncmp(line, "# SDF-EOH", 9) == 0) {
            if (sha1_chunks < 0) break;
            size = (size_t)std::ftell(f) + (size_t)sha1_chunks * (sizeof(int) + 20);
            return ADECO_OK;
        }
    }
    return fail(ADECO_ERR_ARGUMENT, "failed to parse the SDF header");
}

// two pinned buffers; chunk k is read into one while chunk k-1 is copied and decoded from the other
struct ChunkPipe {
    unsigned char *host[2] = {nullptr, nullptr};
    unsigned char *dev[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    ~ChunkPipe()
    {
        for (int b = 0; b < 2; ++b) {
            if (host[b]) cudaFreeHost(host[b]);
            if (dev[b]) cudaFree(dev[b]);
            if (done[b]) cudaEventDestroy(done[b]);
        }
    }
    int open()
    {
        for (int b = 0; b < 2; ++b) {
            CUDA_TRY(cudaMallocHost(&host[b], kReadChunk));
            CUDA_TRY(cudaMalloc(&dev[b], kReadChunk));
            CUDA_TRY(cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming));
        }
        return ADECO_OK;
    }
};

}  // namespace adeco
