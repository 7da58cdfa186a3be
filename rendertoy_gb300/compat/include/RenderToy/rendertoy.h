// RenderToy/rendertoy.h — umbrella header of the RenderToy-compatible API.
#ifndef RTX_COMPAT_RENDERTOY_H
#define RTX_COMPAT_RENDERTOY_H
#include "bvh.h"
#include "compositor.h"
#include "exception.h"
#include "exporter.h"
#include "importer.h"
#include "material.h"
#include "object.h"
#include "ray.h"
#include "renderer.h"
#include "rtmath.h"
#include "world.h"
#endif
