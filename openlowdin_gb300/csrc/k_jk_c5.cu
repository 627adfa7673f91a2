// J/K kernels (FP64 and FP32) of bra pair class 5 (dd) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_JK_TABLES(5)
}  // namespace lgb
