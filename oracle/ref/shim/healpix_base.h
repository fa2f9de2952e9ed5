#include "shim_common.h"
