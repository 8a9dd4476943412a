// Shim for libcgls's scene.h: handle types named in reference declarations.
// Test infrastructure only.
#pragma once
struct scene_ref { int id; };
struct texture_ref { int id; };
