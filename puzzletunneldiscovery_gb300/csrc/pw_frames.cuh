// pw_frames.cuh -- the frames a state is written in, for host and device code.
//
// The unit frame (translateToUnitState / translateFromUnitState,
// lib/osr/unit_world.cc:526-554, with applyPertubation / unapplyPertubation,
// :713-737) and the OMPL frame (translateOMPLStateToUnitState, :689-711).
// Every operation goes through pw_math.cuh's separately rounded helpers, so a
// state converted on the device equals the same state converted by the
// library's host entry points bit for bit.
#pragma once

#include "pw_math.cuh"

namespace pwfr {

// What a conversion needs from a world, as doubles.
struct Frame {
	double scale;     // the scene's scale to the unit frame
	double pert[7];   // the perturbation state (identity: 0 0 0 1 0 0 0)
	double dc[3];     // (OMPL centre - centre of the robot) * scale
};

// Hamilton product a * b, quaternions (w, x, y, z).
PW_HD void quat_mul(const double *a, const double *b, double *o) { pwm::quat_mul(a, b, o); }

PW_HD void mat_vec(const double *R, const double *v, double *o)
{
	for (int i = 0; i < 3; i++)
		o[i] = pwm::add(pwm::add(pwm::mul(R[3 * i], v[0]), pwm::mul(R[3 * i + 1], v[1])), pwm::mul(R[3 * i + 2], v[2]));
}

// decompose (osr_state.cc:85-92): translation and normalised rotation.
PW_HD void decompose(const double *q, double *t, double *rot)
{
	t[0] = q[0]; t[1] = q[1]; t[2] = q[2];
	const double r[4] = { q[3], q[4], q[5], q[6] };
	pwm::quat_normalize(r, rot);
}

// compose (osr_state.cc:107-119): the rotation is normalised again.
PW_HD void compose(const double *t, const double *rot, double *q)
{
	double r[4];
	pwm::quat_normalize(rot, r);
	q[0] = t[0]; q[1] = t[1]; q[2] = t[2];
	q[3] = r[0]; q[4] = r[1]; q[5] = r[2]; q[6] = r[3];
}

// applyPertubation (unit_world.cc:713-724).
PW_HD void apply_pert(const double *pert, const double *in, double *out)
{
	double t[3], rot[4], pt[3], prot[4], qret[4], R[9], Rt[3], tret[3];
	decompose(in, t, rot);
	decompose(pert, pt, prot);
	quat_mul(prot, rot, qret);
	pwm::quat_to_matrix(prot, R);
	mat_vec(R, t, Rt);
	for (int c = 0; c < 3; c++) tret[c] = pwm::add(pt[c], Rt[c]);
	compose(tret, qret, out);
}

// unapplyPertubation (unit_world.cc:726-737).
PW_HD void unapply_pert(const double *pert, const double *in, double *out)
{
	using namespace pwm;
	double t[3], rot[4], pt[3], prot[4], inv[4], R[9], d[3], tret[3], qret[4];
	decompose(in, t, rot);
	decompose(pert, pt, prot);
	const double n2 = add(add(add(mul(prot[1], prot[1]), mul(prot[2], prot[2])), mul(prot[3], prot[3])),
	                      mul(prot[0], prot[0]));
	inv[0] = dvd(prot[0], n2); inv[1] = dvd(-prot[1], n2); inv[2] = dvd(-prot[2], n2); inv[3] = dvd(-prot[3], n2);
	quat_to_matrix(inv, R);
	for (int c = 0; c < 3; c++) d[c] = add(-pt[c], t[c]);
	mat_vec(R, d, tret);
	quat_mul(inv, rot, qret);
	compose(tret, qret, out);
}

// translateToUnitState (unit_world.cc:526-539): scale, then perturb.
PW_HD void to_unit(const Frame &F, const double *in, double *out)
{
	double tmp[7];
	for (int c = 0; c < 3; c++) tmp[c] = pwm::mul(F.scale, in[c]);
	for (int c = 3; c < 7; c++) tmp[c] = in[c];
	apply_pert(F.pert, tmp, out);
}

// translateFromUnitState (unit_world.cc:541-554).
PW_HD void from_unit(const Frame &F, const double *in, double *out)
{
	double tmp[7];
	unapply_pert(F.pert, in, tmp);
	const double inv = pwm::dvd(1.0, F.scale);
	for (int c = 0; c < 3; c++) out[c] = pwm::mul(inv, tmp[c]);
	for (int c = 3; c < 7; c++) out[c] = tmp[c];
}

// translateOMPLStateToUnitState (unit_world.cc:689-711) of one OMPL state
// (x, y, z, qx, qy, qz, qw): w-last to w-first, to the unit frame, then
// t' = t - R(q) * dc.
PW_HD void ompl_to_unit(const Frame &F, const double *p, double *out)
{
	const double wf[7] = { p[0], p[1], p[2], p[6], p[3], p[4], p[5] };
	double u[7], t[3], rot[4], R[9], Rd[3], t2[3];
	to_unit(F, wf, u);
	decompose(u, t, rot);
	pwm::quat_to_matrix(rot, R);
	mat_vec(R, F.dc, Rd);
	for (int c = 0; c < 3; c++) t2[c] = pwm::sub(t[c], Rd[c]);
	compose(t2, rot, out);
}

} // namespace pwfr
