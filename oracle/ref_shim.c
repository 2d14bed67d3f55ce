/* Definition for the stand-in declared in ref_shim.h. */
unsigned char mmc_core_cl[1] = {0};
