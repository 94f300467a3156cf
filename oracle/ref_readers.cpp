// ref_readers.cpp -- C entry point over the reference's own particle readers,
// compiled from the reference sources (with the single-rank MPI stand-in in
// oracle/mpi_stub) into oracle/_ref/libadeco_ref_readers.so.  TEST
// INFRASTRUCTURE ONLY: it makes the golden reader fixtures; nothing in the
// product loads it.
//
// Calls made:
//   get_reader(format)->load_data(file, 0, 1, stride)    src/AdPointDataReaders.h:914, :229
//   get_global_bbox_mpi(particles)                       src/AdPointDataReaders.h:136
//   apply_boundary_corrections(bbox, dims, ColumnMajorOrder, particles)
//                                                        src/AdPointDataReaders.h:155
// The particles are then placed at their linear ids (x fastest), as the
// single-rank redistribution does (src/AdDepositWorkFlow.h:127-137).
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <vector>

#include "AdPointDataReaders.h"

using namespace AdaptiveMassDeposit;

extern "C" int ref_read_particles(const char *path, const char *format, int stride, int periodic, float *xyz,
                                  long long capacity, int dims_out[3], float bbox_out[6])
{
    try {
        std::shared_ptr<AdPointDataReader> reader = get_reader(format);
        reader->load_data(path, 0, 1, stride);
        const AvVec3i dims = reader->get_global_particle_dims();
        const AABBox bbox = get_global_bbox_mpi(reader->get_particles_per_rank());
        if (periodic) {
            ColumnMajorOrder idc;
            apply_boundary_corrections(bbox, dims, idc, *(reader->get_particles_per_rank()[0]));
        }
        for (int a = 0; a < 3; ++a) {
            dims_out[a] = dims[a];
            bbox_out[2 * a] = bbox.min[a];
            bbox_out[2 * a + 1] = bbox.max[a];
        }
        particles_with_ids_chunk &p = *(reader->get_particles_per_rank()[0]);
        const long long n = (long long)dims[0] * dims[1] * dims[2];
        if (n > capacity) return -2;
        const Particles::pos_t_vec &px = *p.get_positions(0), &py = *p.get_positions(1), &pz = *p.get_positions(2);
        const Particles::ids_t_vec &ids = *p.get_ids();
        for (size_t i = 0; i < p.get_num(); ++i) {
            const long long id = (long long)ids[i];
            if (id < 0 || id >= n) return -3;
            xyz[3 * id] = px[i];
            xyz[3 * id + 1] = py[i];
            xyz[3 * id + 2] = pz[i];
        }
        return 0;
    } catch (...) {
        return -1;
    }
}
