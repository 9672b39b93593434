// Stub of stb_image_write for building the reference CPU generator without
// image I/O.  TEST INFRASTRUCTURE ONLY (oracle/_ref build).
#pragma once
inline int stbi_write_tga(const char*, int, int, int, const void*) { return 0; }
