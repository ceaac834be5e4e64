/* Test-infrastructure shim: the libmol2 vector type and macros used by the
 * reference (src/index.c:40-43, src/saxs_utils.c:10).  libmol2 is absent here. */
#ifndef SXS_SHIM_MOL2_VECTOR_H
#define SXS_SHIM_MOL2_VECTOR_H
struct mol_vector3 { double X, Y, Z; };
#define MOL_VEC_ADD(d, a, b) do { (d).X = (a).X + (b).X; (d).Y = (a).Y + (b).Y; (d).Z = (a).Z + (b).Z; } while (0)
#define MOL_VEC_SUB(d, a, b) do { (d).X = (a).X - (b).X; (d).Y = (a).Y - (b).Y; (d).Z = (a).Z - (b).Z; } while (0)
#define MOL_VEC_MULT_SCALAR(d, a, s) do { (d).X = (a).X * (s); (d).Y = (a).Y * (s); (d).Z = (a).Z * (s); } while (0)
#define MOL_VEC_SQ_NORM(a) ((a).X * (a).X + (a).Y * (a).Y + (a).Z * (a).Z)
#define MOL_VEC_EUCLIDEAN_DIST_SQ(a, b) (((a).X - (b).X) * ((a).X - (b).X) + ((a).Y - (b).Y) * ((a).Y - (b).Y) + ((a).Z - (b).Z) * ((a).Z - (b).Z))
#endif
