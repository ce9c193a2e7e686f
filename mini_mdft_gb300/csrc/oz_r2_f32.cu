// oz_r2_f32.cu -- the mrso = 2 split lane kernel for float storage and
// arithmetic (the mixed form).
#include "oz_r2.cuh"

MDFT_OZ_R2_INSTANTIATE(float, 1)
MDFT_OZ_R2_INSTANTIATE(float, 2)
MDFT_OZ_R2_INSTANTIATE(float, 3)
MDFT_OZ_R2_INSTANTIATE(float, 4)
MDFT_OZ_R2_INSTANTIATE(float, 5)
MDFT_OZ_R2_INSTANTIATE(float, 6)
