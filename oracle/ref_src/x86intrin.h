/* Empty stand-in: the reference's vectorization.h includes <x86intrin.h>
 * unconditionally; with the ISA macros undefined it then uses its generic
 * one-lane VectorizedArray (vectorization.h:34-158), so the reference's
 * lane-interleaved DG layout becomes the plain cell-major layout. */
