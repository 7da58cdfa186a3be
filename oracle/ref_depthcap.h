/*
 * ref_depthcap.h — force-included into the reference sources by
 * oracle/Makefile (target `ref`).  The build-time copy of RenderToy's
 * src/renderer.cpp replaces the literal recursion cap `depth > 4`
 * (renderer.cpp:274) by `depth > rtx_ref_depth_cap`; that is the only change
 * made to the reference, and a cap of 4 reproduces the unmodified build
 * (checked by tests/golden/make_golden.py).  TEST INFRASTRUCTURE ONLY.
 */
#ifndef RTX_REF_DEPTHCAP_H
#define RTX_REF_DEPTHCAP_H
extern int rtx_ref_depth_cap;
#endif
