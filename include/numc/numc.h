/* Umbrella header of the numc-compatible GB300 library (numc's
 * include/numc/numc.h:12-21 includes the same set minus cuda.h). */
#ifndef NUMC_NUMC_H
#define NUMC_NUMC_H

#include "numc/export.h"
#include "numc/dtype.h"
#include "numc/error.h"
#include "numc/array.h"
#include "numc/math.h"
#include "numc/random.h"
#include "numc/cuda.h"

#endif /* NUMC_NUMC_H */
