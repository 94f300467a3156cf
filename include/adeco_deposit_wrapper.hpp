// adeco_deposit_wrapper.hpp -- drop-in C++ replacement for ADECO's
// AdaptiveMassDeposit::DepositWrapper (src/AdDeposit2Grid.h:59-93), header
// only, over the C ABI of libadeco_gb300.so.
//
// Same signature, argument meaning and error behaviour as the reference:
// the result is ACCUMULATED into `data`, an empty input returns silently,
// and every failure throws AdRuntimeException (a std::exception) -- where the
// reference's CUDA path would exit(EXIT_FAILURE) on a CUDA error
// (src/AdDeposit2Grid.cu:59-76), this one throws too.
#ifndef ADECO_DEPOSIT_WRAPPER_HPP
#define ADECO_DEPOSIT_WRAPPER_HPP

#include <cstddef>
#include <stdexcept>
#include <string>

#include "adeco_deposit.h"

#define AMD_CUDA_BLOCK_DIM 64
#define AMD_CUDA_GRID_DIM 512

namespace AdaptiveMassDeposit {

class AdRuntimeException : public std::runtime_error {
public:
    AdRuntimeException(const std::string &msg, int code = ADECO_ERR_ARGUMENT) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

class DepositWrapper {
public:
    typedef float h_grid_mass_type;
    typedef float vertex_type;
    typedef float mass_type;

    // launch geometry is chosen per device by the library; kept for source compatibility
    static inline int get_cuda_grid_size() { return AMD_CUDA_GRID_DIM; }
    static inline int get_cuda_block_size() { return AMD_CUDA_BLOCK_DIM; }

    static void deposit_tets(const bool use_specific_gpu, const size_t device_id_to_use, const size_t tet_offset,
                             const size_t num_tets_2_process, const float *positions, const size_t positions_size,
                             const int meta_cells_per_patch, const float bbox[6], const int dims,
                             h_grid_mass_type *data)
    {
        const int rc = adeco_deposit_tets(use_specific_gpu ? 1 : 0, device_id_to_use, tet_offset, num_tets_2_process,
                                          positions, positions_size, meta_cells_per_patch, bbox, dims, data);
        if (rc != ADECO_OK)
            throw AdRuntimeException(std::string("ERROR: deposit_tets(): ") + adeco_last_error(), rc);
    }
};

}  // namespace AdaptiveMassDeposit

#endif
