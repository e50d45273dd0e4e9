// Included by the reference host beside xrt_kernel.h; the stand-in types live there.
#pragma once
#include "xrt_kernel.h"
