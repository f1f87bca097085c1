/*
 * ref_config.h -- TEST INFRASTRUCTURE. Build configuration for compiling the
 * reference ODE 0.12 sources into oracle/_ref/ (see oracle/Makefile). It is
 * force-included ahead of every reference translation unit and claims the
 * reference's own config.h include guard, so that file's trimesh/OPCODE
 * settings are not used: the path under test needs no trimesh, libccd, OU or
 * TLS. The settings below are the ones the remaining sources consult.
 */
#ifndef _ODE_CONFIG_H_
#define _ODE_CONFIG_H_
#define dTRIMESH_ENABLED 0
#define dTRIMESH_OPCODE 0
#define dTRIMESH_GIMPACT 0
#define dTRIMESH_16BIT_INDICES 0
#define dTRIMESH_OPCODE_USE_OLD_TRIMESH_TRIMESH_COLLIDER 0
#define ODE_PLATFORM_LINUX
#include <malloc.h>
#include <alloca.h>
#include <float.h>
#include <stddef.h>
#ifdef dSINGLE
#define dEpsilon FLT_EPSILON
#else
#define dEpsilon DBL_EPSILON
#endif
typedef size_t intP;
#define EFFICIENT_ALIGNMENT 16
#endif
