// coupling kernels (FP64 and FP32) of bra pair class 1 (ps) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_CP_TABLES(1)
}  // namespace lgb
