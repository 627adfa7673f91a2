// J/K kernels (FP64 and FP32) of bra pair class 4 (dp) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_JK_TABLES(4)
}  // namespace lgb
