"""Rigid kinematics of a cut body for mge_move_surface, standing in for the
displacements, normals and velocities the reference's FSI framework hands
to movsurf.f90: every record's surface point turned by theta about the z
axis through the centre and shifted by (0, y, 0), its normal turned with it,
and its velocity that of the rigid motion (turning rate dtheta, heave rate
dy, in the solver's velocity units) times vel_fs."""
import numpy as np

# input_param.f90:51, vel_fs = rm*sqrt(gamma*gas_pmean/gas_rhomean), for
# M = 0.3 in sea-level air
VEL_FS = 0.3 * np.sqrt(1.4 * 101325.0 / 1.225)


def rigid(spec, theta, y=0.0, dtheta=0.0, dy=0.0, vel_fs=VEL_FS, center=(0.0, 0.0, 0.0)):
    """(disp, norv, vel) for the records of one block spec, [nmir, 3] each."""
    a = spec.arrays
    ps = np.asarray(a["psurf"], dtype=np.float64).reshape(-1, 3)
    nv = np.asarray(a["nvec"], dtype=np.float64).reshape(-1, 3)
    c = np.asarray(center, dtype=np.float64)
    ct, st = np.cos(theta), np.sin(theta)
    R = np.array([[ct, -st, 0.0], [st, ct, 0.0], [0.0, 0.0, 1.0]])
    r = (ps - c) @ R.T
    disp = c + r + np.array([0.0, y, 0.0]) - ps
    norv = nv @ R.T
    vel = np.zeros_like(ps)
    vel[:, 0] = -dtheta * r[:, 1]
    vel[:, 1] = dtheta * r[:, 0] + dy
    return disp, norv, vel * vel_fs


def move_all(cyc, case, **kw):
    """One rigid motion on every block of every level that has records."""
    for L, specs in enumerate(case.levels, start=1):
        for s, sp in enumerate(specs, start=1):
            if sp.arrays and sp.arrays["nmir"]:
                cyc.move_surface(L, *rigid(sp, **kw), vel_fs=kw.get("vel_fs", VEL_FS), serial=s)
