// Serving loop types shared with the C ABI header.
#pragma once
#include "../../include/fastpcc_gb300.h"
