// oz_r2_df.cu -- the mrso = 2 split lane kernel for packed double-float
// storage and arithmetic.
#include "oz_r2.cuh"

MDFT_OZ_R2_INSTANTIATE(mdft::DF, 1)
MDFT_OZ_R2_INSTANTIATE(mdft::DF, 2)
MDFT_OZ_R2_INSTANTIATE(mdft::DF, 3)
MDFT_OZ_R2_INSTANTIATE(mdft::DF, 4)
MDFT_OZ_R2_INSTANTIATE(mdft::DF, 5)
MDFT_OZ_R2_INSTANTIATE(mdft::DF, 6)
