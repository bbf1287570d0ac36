"""GB300-native HorseIR builtin library (libhgpu.so) and its Python binding."""
