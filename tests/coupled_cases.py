"""Problems of two coupled scalar fields (FG_PROBLEM_COUPLED) shared by the
CPU and GPU tests: u and v, coupled both ways (mass with a point
coefficient and advection from u into v's rows, grad-grad from v into
u's rows)."""


def coupled_configs(F):
    C = F.FG_PROBLEM_COUPLED
    return {
        # same-order Lagrange fields with u fixed on the boundary: the lifting
        # of the fixed u DOFs into v's rows through the coupling block
        "tri_lagrange_p2_dirichlet": F.config(kind=C, dim=2, m=5, mesh_order=2, space=F.FG_SPACE_LAGRANGE, gauss=4, jitter=0.2,
                                              seed=3, k=3.0, dirichlet=1, dirichlet_value=1.0, source=1),
        # different orders: 10 x 6 and 6 x 10 element blocks, bubbles in u
        "tri_h1_p3_p2": F.config(kind=C, dim=2, m=4, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=3, order2=2, gauss=6,
                                 jitter=0.2, seed=4, k=3.0, source=1),
        "tet_h1_p2_p1": F.config(kind=C, dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=2, order2=1, gauss=4,
                                 jitter=0.15, seed=3, k=3.0),
        "tet_h1_p1_p3": F.config(kind=C, dim=3, m=2, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=1, order2=3, gauss=6,
                                 jitter=0.15, seed=5, k=2.0, source=1),
    }


def lifting_undefined_config(F):
    """u (order 1) fixed on the boundary, v of order 2: the block (v rows, u
    columns) has 6 x 3 entries, and the lifting read of addValuesDC,
    values[j * 3 + i] for i < 6, j < 3, is not the transposed entry."""
    return F.config(kind=F.FG_PROBLEM_COUPLED, dim=2, m=3, mesh_order=1, space=F.FG_SPACE_HIERARCHICAL_H1, order=1, order2=2,
                    gauss=4, jitter=0.2, seed=2, k=2.0, dirichlet=1, dirichlet_value=1.0)
