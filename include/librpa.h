#pragma once
/*
 * Aggregate header (replaces LibRPA include/librpa.h:19-31).
 */
#include "librpa_global.h"
#include "librpa_input.h"
#include "librpa_compute.h"
#include "librpa_gb300.h"
