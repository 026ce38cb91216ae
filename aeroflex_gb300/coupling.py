"""Static aeroelastic coupling of the residual path to the structure module's
beam: the loop the reference's coupler sketches (rans.h:99-102 hands the
wall forces of each converged solve to the aerodynamic database,
model.hpp:94-100 takes a new load vector for the beam), run here on one
airfoil section with the adjoint gradients driving the update.

- Beam: Euler-Bernoulli elements along the chord, two degrees of freedom
  per node (deflection w, slope dw/dx): the bending block of the structure
  module's bar element (element.hpp:77-110: 12EI/L^3, 6EI/L^2, 4EI/L,
  2EI/L), assembled as MODEL::set_K_global does, clamped as
  set_K_Final_sparse does (constrained rows and columns zeroed, unit
  diagonal, load zeroed), loaded through set_load_vector_from_vector
  (model.hpp:94-100: a vector of another size is ignored) and solved
  directly (get_Lin_Solve).
- Loads: per wall face the pressure force per unit span,
  q_inf * c * cp * n_y * L (n the face normal into the body, L the face
  length in chords): the face sums of the force integration
  (post.h:341-375), lumped onto the beam by its cubic shape functions at the
  face centre.
- Shape: the deflection w(x) moves wall node k vertically by w(x_k) / c
  (chords), spread into the volume by inverse-distance weighting
  (afx_deform_patch_xy): upper and lower surface move together, the
  trailing edge with them.
- Flow: each shape converged by the solver's implicit iteration, then its
  Newton-Krylov finish (afx_newton_solve) to a tight tolerance, so the
  adjoint is taken at the discrete steady state.
- Update: Newton on K u = F(u) with the load Jacobian taken from the
  adjoint as rank one, F(u) ~ F_n + s g.(u - u_n): s = F_n / C_y,n (the load
  shape per unit normal-force coefficient) and
  g = dC_y/du = cos(alpha) dC_L/du + sin(alpha) dC_D/du, where dJ/du_j is
  the adjoint shape derivative along beam mode j's surface displacement
  (afx_adjoint_patch_dirs_xy).  The rank-one system is solved by
  Sherman-Morrison.  dC_D/du also predicts each step's drag change and
  dC_L/dalpha turns the lift change into an equivalent angle; both are
  recorded beside the changes the next flow solve gives.
"""
import math

import numpy as np

from . import rans


class Beam:
    """Cantilever of ``n_elem`` equal Euler-Bernoulli elements on
    [x0, x0 + length] (metres), bending stiffness ``EI`` (N m^2 per metre of
    span), clamped at x0.  Degrees of freedom: (w_i, theta_i) per node."""

    def __init__(self, n_elem=50, EI=1e4, length=1.0, x0=0.0):
        self.n_elem, self.EI, self.length, self.x0 = int(n_elem), float(EI), float(length), float(x0)
        self.n_nodes = self.n_elem + 1
        self.n_dof = 2 * self.n_nodes
        self.xn = x0 + length * np.arange(self.n_nodes) / self.n_elem
        Le = length / self.n_elem
        k = self.EI / Le ** 3 * np.array([[12.0, 6 * Le, -12.0, 6 * Le],
                                          [6 * Le, 4 * Le * Le, -6 * Le, 2 * Le * Le],
                                          [-12.0, -6 * Le, 12.0, -6 * Le],
                                          [6 * Le, 2 * Le * Le, -6 * Le, 4 * Le * Le]])
        K = np.zeros((self.n_dof, self.n_dof))
        for e in range(self.n_elem):
            s = slice(2 * e, 2 * e + 4)
            K[s, s] += k
        self.K_global = K
        self.clamped = np.array([0, 1])  # w and theta at x0
        Kf = K.copy()
        Kf[self.clamped, :] = 0.0
        Kf[:, self.clamped] = 0.0
        Kf[self.clamped, self.clamped] = 1.0
        self.K_final = Kf
        self.forces = np.zeros(self.n_dof)

    def set_load_vector_from_vector(self, f):
        """Replaces the load vector when the size matches; returns whether it
        did (model.hpp:94-100 ignores a vector of another size)."""
        f = np.asarray(f, np.float64)
        if f.shape != self.forces.shape:
            return False
        self.forces = f.copy()
        return True

    def apply_spc(self, f):
        f = np.array(f, np.float64)
        f[self.clamped] = 0.0
        return f

    def solve(self, f=None):
        """Displacements of load vector f (the stored one when None)."""
        return np.linalg.solve(self.K_final, self.apply_spc(self.forces if f is None else f))

    def shape_matrix(self, x):
        """N (len(x), n_dof): w(x) = N @ u, cubic Hermite on each element
        (x clipped to the beam)."""
        x = np.clip(np.asarray(x, np.float64), self.x0, self.x0 + self.length)
        Le = self.length / self.n_elem
        e = np.minimum(((x - self.x0) / Le).astype(np.int64), self.n_elem - 1)
        xi = (x - self.x0 - e * Le) / Le
        N = np.zeros((len(x), self.n_dof))
        r = np.arange(len(x))
        N[r, 2 * e] = 1 - 3 * xi ** 2 + 2 * xi ** 3
        N[r, 2 * e + 1] = Le * (xi - 2 * xi ** 2 + xi ** 3)
        N[r, 2 * e + 2] = 3 * xi ** 2 - 2 * xi ** 3
        N[r, 2 * e + 3] = Le * (xi ** 3 - xi ** 2)
        return N


def rank_one_newton(beam, F, s, g, u):
    """Solution of K x = F + s g.(x - u) (the beam with loads linearised
    about state u as F + s g.(x - u)) by Sherman-Morrison:
    x = y1 + y2 (g.y1) / (1 - g.y2), y1 = K^-1 (F - s g.u), y2 = K^-1 s."""
    y1 = beam.solve(F - s * float(g @ u))
    y2 = beam.solve(s)
    return y1 + y2 * float(g @ y1) / (1.0 - float(g @ y2))


def sea_level_dynamic_pressure(mach, rho=1.225, a=340.294):
    """q_inf = rho (M a)^2 / 2 in Pa at the standard sea-level density and
    speed of sound."""
    v = mach * a
    return 0.5 * rho * v * v


class Coupling:
    """Aeroelastic loop on an FP64 solver's wall patch.

    ``solver`` (rans.Solver, fp64, not Spalart-Allmaras: the adjoint covers
    the inviscid and laminar fluxes) is initialised; ``mesh_arrays`` are the
    arrays its mesh was made from (node coordinates, undeformed);
    ``mesh`` is the rans.mesh made from them (edge and boundary numbering).
    The beam spans the chord from the leading edge (chord ``chord_m``
    metres); ``q_inf`` in Pa."""

    def __init__(self, solver, mesh, mesh_arrays, beam, q_inf, chord_m=1.0, patch="wall", tol=1e-12,
                 switch_tol=1e-6, max_it=400, adjoint_tol=1e-12, adjoint_max_it=600, h=1e-7, flow_solver=None,
                 newton_cfl=0.0):
        self.s, self.beam, self.q_inf, self.c, self.patch = solver, beam, float(q_inf), float(chord_m), patch
        self.tol, self.switch_tol, self.max_it = tol, switch_tol, max_it
        self.adj_tol, self.adj_max_it, self.h = adjoint_tol, adjoint_max_it, h
        # the primal may run on another solver of the same mesh (an
        # FP32-mixed one: FP64 right-hand side and update, so the same
        # converged state), the adjoint always on `solver` (FP64)
        self.fs = flow_solver if flow_solver is not None else solver
        self.newton_cfl = newton_cfl
        ids, nx, ny = solver.patch_nodes(patch)
        self.ids, self.pnx, self.pny = ids, nx, ny
        x0 = np.asarray(mesh_arrays["x"], np.float64)
        y0 = np.asarray(mesh_arrays["y"], np.float64)
        self.x0, self.y0 = x0, y0
        # wall faces in the order of the force integration (boundary order)
        names = mesh.boundary_names()
        be = mesh.get_int("boundary_edges")
        en = mesh.get_int("edges_nodes").reshape(-1, 2)
        wall = np.array([n == patch for n in names])
        self.face_nodes = en[be[wall]]
        pos = np.full(len(x0), -1, np.int64)
        pos[ids] = np.arange(len(ids))
        if (pos[self.face_nodes] < 0).any():
            raise ValueError("wall faces with nodes off the patch")
        self.face_pos = pos[self.face_nodes]
        # orientation of (dy, -dx) along each face's node order against the
        # mesh's normal (out of the fluid, into the body): fixed by topology
        self.orient = np.ones(len(self.face_nodes))
        _, nx0, ny0, _ = self.wall_faces(np.zeros(len(ids)))
        self.orient = np.sign(nx0 * mesh.get("nx")[be[wall]] + ny0 * mesh.get("ny")[be[wall]])
        xs = x0[ids] * self.c  # patch nodes along the beam (undeformed)
        self.T = beam.shape_matrix(xs) / self.c  # vertical displacement dy = T u (chords per metre / radian)
        self.free = np.setdiff1d(np.arange(beam.n_dof), beam.clamped)
        self.u = np.zeros(beam.n_dof)
        self.history = []

    def surface_displacement(self, u):
        """Vertical displacement of each patch node (chords)."""
        return self.T @ u

    def wall_faces(self, a):
        """(x_centre, n_x, n_y, length) of the wall faces with the patch
        nodes displaced vertically by a: the solver's own face metrics."""
        px = self.x0[self.ids]
        py = self.y0[self.ids] + a
        p0, p1 = self.face_pos[:, 0], self.face_pos[:, 1]
        dx, dy = px[p1] - px[p0], py[p1] - py[p0]
        L = np.sqrt(dx * dx + dy * dy)
        nx, ny = self.orient * dy / L, -self.orient * dx / L
        xc = 0.5 * (px[p0] + px[p1])
        return xc, nx, ny, L

    def loads(self, a, cp):
        """(load vector on the beam (N, N m per metre of span), C_y from
        the same face sums with the force integration's normalisation)."""
        xc, nx, ny, L = self.wall_faces(a)
        fy = cp * ny * L
        F = self.beam.shape_matrix(xc * self.c).T @ (self.q_inf * self.c * fy)
        return F, float(fy.sum() / (xc.max() - xc.min()))

    def _gradient(self, objective):
        (da, dM), it, res = self.s.adjoint_solve(self.patch, objective, tol=self.adj_tol, max_it=self.adj_max_it)
        dirs = np.zeros((len(self.free), len(self.ids), 2))
        dirs[:, :, 1] = self.T[:, self.free].T
        g = np.zeros(self.beam.n_dof)
        g[self.free] = self.s.adjoint_patch_dirs_xy(dirs, self.patch, objective, h=self.h)
        return g, da, dict(iterations=it, residual=res)

    def flow(self, u):
        """Flow on the shape of beam state u: the implicit iteration to
        switch_tol, then the Newton-Krylov finish to tol.  Returns (a,
        dict of implicit iterations, Newton and Krylov steps, err, wall
        profile)."""
        a = self.surface_displacement(u)
        for g in {id(self.s): self.s, id(self.fs): self.fs}.values():
            g.deform_patch_xy(np.zeros_like(a), a, self.patch)
        it, err = self.fs.run_solver(self.switch_tol, self.max_it)
        nn, nk, err = self.fs.newton_solve(self.tol, 30, self.newton_cfl)
        if self.fs is not self.s:
            self.s.set_q(self.fs.get_q())
        w = rans.get_wall_profile(self.s, self.patch)
        return a, dict(implicit=it, newton=nn, krylov=nk), err, w

    def step(self, alpha):
        """One coupling iteration from the current beam state: flow solve on
        the deformed shape, loads, both adjoints, Newton update.  Returns the
        history entry."""
        u = self.u
        a, it, err, w = self.flow(u)
        F, cy = self.loads(a, w["cp"])
        gL, dcl_da, infL = self._gradient("cl")
        gD, dcd_da, infD = self._gradient("cd")
        ca, sa = math.cos(alpha), math.sin(alpha)
        gY = ca * gL + sa * gD
        u_new = rank_one_newton(self.beam, F, F / cy, gY, u)
        du = u_new - u
        self.beam.set_load_vector_from_vector(F)
        e = dict(cl=w["cl"], cd=w["cd"], cm=w["cm"], cy=cy, cy_solver=ca * w["cl"] + sa * w["cd"],
                 flow_iterations=it, flow_residual=err, adjoint_cl=infL, adjoint_cd=infD,
                 dcl_dalpha=dcl_da, dcd_dalpha=dcd_da, tip_deflection_m=float(u[2 * self.beam.n_elem]),
                 max_surface_displacement=float(np.abs(a).max()), load_N_per_m=float(F[0::2].sum()),
                 dcl_pred=float(gL @ du), dcd_pred=float(gD @ du),
                 alpha_equivalent_deg=math.degrees(float(gL @ du) / dcl_da) if dcl_da else None,
                 step_norm_m=float(np.abs(du[0::2]).max()))
        self.history.append(e)
        self.u = u_new
        return e

    def run(self, alpha, iterations=5):
        """``iterations`` coupling steps, then the flow on the final shape
        (its C_L, C_D close the last step's prediction)."""
        for _ in range(iterations):
            self.step(alpha)
        a, it, err, w = self.flow(self.u)
        final = dict(cl=w["cl"], cd=w["cd"], cm=w["cm"], flow_iterations=it, flow_residual=err,
                     tip_deflection_m=float(self.u[2 * self.beam.n_elem]))
        return self.history, final
