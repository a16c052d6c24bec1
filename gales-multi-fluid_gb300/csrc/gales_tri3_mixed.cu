// Kernel instances for the tri3 element (dim 2, 3 nodes, 3 interior points,
// 3 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tri3_mixed() { return InteriorDispatch<2, 3, 3, GALES_FORM_MIXED>::ops(); }

}  // namespace gales
