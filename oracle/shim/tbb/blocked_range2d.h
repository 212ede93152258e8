// Scheduling-name stand-in: everything lives in tbb.h beside this file.
#pragma once
#include "tbb.h"
