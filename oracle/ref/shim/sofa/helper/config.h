// Stand-in for sofa/helper/config.h (oracle reference harness only).
#pragma once
#include <sofa/config.h>
#define SOFA_HELPER_API
