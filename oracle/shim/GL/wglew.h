/* Test infrastructure (oracle only): headless stand-in for the WGL extension header. */
#ifndef OC_SHIM_WGLEW_H
#define OC_SHIM_WGLEW_H
#include "glew.h"
#define wglSwapIntervalEXT(...) (0)
#endif
