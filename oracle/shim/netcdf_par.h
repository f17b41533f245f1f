/* Parallel netCDF declarations are not needed by the single-rank oracle. */
#pragma once
#include "netcdf.h"
