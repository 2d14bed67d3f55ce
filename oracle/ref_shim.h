/* Forced-include shim for building the reference CPU engine without its
 * embedded OpenCL kernel text: mmc_utils.c compares cfg->clsource against the
 * symbol mmc_core_cl even when MCX_EMBED_CL is off.  A one-byte stand-in makes
 * those comparisons well-defined (clsource stays NULL on the CPU path). */
#ifndef MMCGB_REF_SHIM_H
#define MMCGB_REF_SHIM_H
extern unsigned char mmc_core_cl[];
#endif
