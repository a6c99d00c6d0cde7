/* float variant of the CPU oracle (TEST INFRASTRUCTURE ONLY; see qll_oracle.h) */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "qll_oracle.h"
#define real float
#define S F
#include "oracle_impl.h"
