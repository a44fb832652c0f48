/* Oracle stand-in: every TSQR/Teuchos type the reference names lives in Tsqr.hpp. */
#include "Tsqr.hpp"
