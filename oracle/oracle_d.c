/* double variant of the CPU oracle (TEST INFRASTRUCTURE ONLY; see qll_oracle.h) */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "qll_oracle.h"
#define real double
#define S D
#include "oracle_impl.h"
