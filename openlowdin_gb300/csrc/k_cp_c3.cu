// coupling kernels (FP64 and FP32) of bra pair class 3 (ds) for every ket pair class.
#include "class_tables.cuh"

namespace lgb {
LGB_CP_TABLES(3)
}  // namespace lgb
