#pragma once
/*
 * Enumerations and constants of the LibRPA C API (values kept identical to
 * LibRPA include/librpa_enums.h so that callers and the Fortran binding see
 * the same numbers).
 */
#ifdef __cplusplus
extern "C" {
#endif

#define LIBRPA_UNSET -101
#define LIBRPA_AUTO -51
#define LIBRPA_SWITCH_OFF 0
#define LIBRPA_SWITCH_ON 1

#define LIBRPA_VERBOSE_DEBUG 4
#define LIBRPA_VERBOSE_WARN 3
#define LIBRPA_VERBOSE_INFO 2
#define LIBRPA_VERBOSE_CRITICAL 1
#define LIBRPA_VERBOSE_SILENT 0

/* Parallel routing (librpa_enums.h:57-64).  This build runs every routing as
 * the same single-GPU block schedule; the value is still validated and reported. */
#define LIBRPA_ROUTING_COUNT 5
typedef enum
{
    ROUTING_UNSET = LIBRPA_UNSET,
    AUTO = LIBRPA_AUTO,
    RTAU = 0,
    ATOMPAIR = 1,
    LIBRI = 2
} LibrpaParallelRouting;

/* Time/frequency grid kinds (librpa_enums.h:66-84). */
#define LIBRPA_TFGRID_COUNT 7
typedef enum
{
    TFGRID_UNSET = LIBRPA_UNSET,
    GaussLegendre = 0,
    GaussChebyshevI = 1,
    GaussChebyshevII = 2,
    Minimax = 3,
    EvenSpaced = 4,
    EvenSpaced_TF = 5
} LibrpaTimeFreqGrid;

typedef int LibrpaSwitch;
typedef int LibrpaKind;
typedef int LibrpaVerbose;

#ifdef __cplusplus
}
#endif
