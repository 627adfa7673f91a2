// first-quarter and MP2 transform-input kernels of bra pair class 4 (dp) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_IT_TABLE(4)
}  // namespace lgb
