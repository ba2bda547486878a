/* Headless stand-in for cuda_gl_interop.h: the graphics-interop calls live in templates that
 * the headless driver never instantiates. */
#pragma once
#include <cuda_runtime_api.h>
