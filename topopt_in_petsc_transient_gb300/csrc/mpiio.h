// mpiio.h -- internal interface of the result-file writer (mpiio.cu) used by
// the LinearElasticity object to emit its physics output.
#pragma once
#include <cuda_runtime.h>

#include "../../include/topopt_gb300.h"

namespace topo {

// Queue one dataset (iteration number, point fields, cell fields).  `nodal`
// holds n_nodal DOF-interleaved 3-vectors of nn nodes (3 point fields each),
// `cells` n_cells element arrays; device arrays are read on `s`.
int mpiio_write(topo_mpiio *io, unsigned long long itr, const double *const *nodal, int n_nodal,
                const double *const *cells, int n_cells, int on_device, cudaStream_t s);
int mpiio_point_fields(const topo_mpiio *io);
int mpiio_cell_fields(const topo_mpiio *io);
long long mpiio_points(const topo_mpiio *io);
long long mpiio_cells(const topo_mpiio *io);

}  // namespace topo
