// Hand-written build configuration for compiling the G+Smo reference sources directly with g++
// (header-only template build, double coefficients, int indices). Written for the parity
// oracle only; it replaces the file G+Smo's own build system would produce.
#pragma once
#define GISMO_VERSION "24.8.0"
#define GISMO_MAJOR 24
#define GISMO_MINOR 8
#define GISMO_PATCH 0
#define GISMO_COEFF_TYPE double
#ifndef real_t
#define real_t GISMO_COEFF_TYPE
#endif
#define index_t int
#define short_t short
#define GISMO_DATA_DIR "./"
#define GISMO_SEARCH_PATHS ""
#define GISMO_CONFIG_DIR "./"
#include <gsCore/gsConfigExt.h>
#define EIGEN_DEFAULT_DENSE_INDEX_TYPE index_t
#define EIGEN_DEFAULT_SPARSE_INDEX_TYPE index_t
#define EIGEN_DEFAULT_TO_COL_MAJOR
#define EIGEN_NO_STATIC_ASSERT
