// C entry points over the reference's own Moller triangle test
// (lib/tritri/Moller97d.cc, compiled where it lies by the Makefile's _ref
// target).  Test infrastructure only: the oracle's restatement of the same
// test is checked against these on random and near-degenerate pairs.

int tri_tri_intersect(const double V0[3], const double V1[3], const double V2[3], const double U0[3],
                      const double U1[3], const double U2[3]);
int tri_tri_intersect_with_isectline(const double V0[3], const double V1[3], const double V2[3],
                                     const double U0[3], const double U1[3], const double U2[3], int *coplanar,
                                     double isectpt1[3], double isectpt2[3]);

extern "C" __attribute__((visibility("default"))) int ref_tri_tri(const double *V0, const double *V1,
                                                                   const double *V2, const double *U0,
                                                                   const double *U1, const double *U2)
{
	return tri_tri_intersect(V0, V1, V2, U0, U1, U2);
}

extern "C" __attribute__((visibility("default"))) int ref_tri_tri_isect(const double *V0, const double *V1,
                                                                         const double *V2, const double *U0,
                                                                         const double *U1, const double *U2,
                                                                         int *coplanar, double *p1, double *p2)
{
	return tri_tri_intersect_with_isectline(V0, V1, V2, U0, U1, U2, coplanar, p1, p2);
}
