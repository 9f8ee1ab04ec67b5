"""illume-gb300: GB300-native wavefront path tracer behind the C-ABI of include/illume.h."""
