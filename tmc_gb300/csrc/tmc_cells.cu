#include "tmc_cells.h"
