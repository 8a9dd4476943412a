/* Shim for the reference's autotools config.h (test infrastructure only). */
#pragma once
#define HAVE_LIBOSDINTERFACE 0
#define HAVE_LIBILMIMF 0
