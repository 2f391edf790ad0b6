// Pore seeds, pore propagation, empty-pore removal and watershed (placeholder).
#include "pma_internal.h"

namespace pma {

pma_table* pores(pma_ctx*, const uint8_t*, const uint32_t*, const uint32_t*, pma_dims, pma_stencil,
                 uint32_t*) {
    throw Error(PMA_ERR_INTERNAL, "pma_pores: not available in this build");
}
void remove_empty_pores(pma_ctx*, pma_table*, uint32_t*, pma_dims) {
    throw Error(PMA_ERR_INTERNAL, "pma_remove_empty_pores: not available in this build");
}
pma_table* watershed(pma_ctx*, const pma_table*, const uint32_t*, pma_dims, pma_stencil, uint32_t,
                     uint32_t*) {
    throw Error(PMA_ERR_INTERNAL, "pma_watershed: not available in this build");
}

}  // namespace pma
