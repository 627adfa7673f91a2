// first-quarter and MP2 transform-input kernels of bra pair class 5 (dd) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_IT_TABLE(5)
}  // namespace lgb
