// Shim: BLAS++ util header (enums live in blas.hh).
#include "../blas.hh"
