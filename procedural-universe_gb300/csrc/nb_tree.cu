// placeholder, replaced by the octree build
#include "nb_internal.hpp"
namespace nb {
cudaError_t tree_reserve(nb_sim*) { return cudaSuccess; }
void tree_free(nb_sim*) {}
cudaError_t tree_build(nb_sim*) { return cudaErrorNotSupported; }
cudaError_t tree_forces(nb_sim*) { return cudaErrorNotSupported; }
}
