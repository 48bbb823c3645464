/* Minimal OpenImageIO stand-in for building the reference as a test oracle.
 * Only what the reference's image/texture code names is declared; image I/O
 * is PFM-only (see oiio_shim.cpp). Test infrastructure, not product code. */
#pragma once
#define OIIO_VERSION 20000
