#pragma once
/*
 * Global functions (replaces LibRPA include/librpa_global.h:19-90).
 */
#include "librpa_enums.h"

#ifdef __cplusplus
extern "C" {
#endif

/* librpa_global.h:25 */
const char* librpa_get_build_info(void);
/* librpa_global.h:32-46 */
int librpa_get_major_version(void);
int librpa_get_minor_version(void);
int librpa_get_patch_version(void);

/* librpa_global.h:62 -- defaults as in LibRPA when compiled as C++. */
#ifdef __cplusplus
void librpa_init_global(LibrpaSwitch switch_redirect_stdout = LIBRPA_SWITCH_OFF,
                        const char *redirect_path = "stdout",
                        LibrpaSwitch switch_process_output = LIBRPA_SWITCH_ON);
#else
void librpa_init_global(LibrpaSwitch switch_redirect_stdout, const char *redirect_path,
                        LibrpaSwitch switch_process_output);
#endif

/* librpa_global.h:72 */
void librpa_finalize_global(void);
/* librpa_global.h:80 -- runs a small self-check of the GPU path against built-in values. */
void librpa_test(void);
/* librpa_global.h:88 -- prints the per-stage timer tree of the last calls. */
void librpa_print_profile(void);

#ifdef __cplusplus
}
#endif
