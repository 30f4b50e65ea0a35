/*
 * lusgs.h -- the natural-order ("serial") array LU-SGS entry points, under
 * the header name examples/mpi3d.c:26 includes.  They are declared, with
 * the colored ones, in coloredlusgs.h.
 */
#pragma once

#include "coloredlusgs.h"
