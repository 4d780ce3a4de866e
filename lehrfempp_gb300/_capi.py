"""ctypes declarations of the C-ABI in include/lfg.h.

This is the Python-side binding a caller uses in place of the reference's C++
templates (the C++ facade include/lf_gb300.hpp is the other binding).  Every
function listed in include/lfg.h is declared here; tests check both lists
against the exported symbols of the shared library.
"""
import ctypes as C

c_status = C.c_int
vp = C.c_void_p
i8, i32, i64 = C.c_int8, C.c_int32, C.c_int64
u8 = C.c_uint8
dbl = C.c_double
sz = C.c_size_t
P = C.POINTER


class lfg_triplet(C.Structure):
    _fields_ = [("row", i32), ("col", i32), ("value", dbl)]


class lfg_coeff(C.Structure):
    _fields_ = [("kind", i32), ("func", i32), ("value", dbl), ("data_dev", vp), ("p", dbl * 16)]


class lfg_rd_provider(C.Structure):
    _fields_ = [("alpha", lfg_coeff), ("gamma", lfg_coeff), ("qr_degree_tria", i32), ("qr_degree_quad", i32)]


class lfg_load_provider(C.Structure):
    _fields_ = [("f", lfg_coeff), ("qr_degree_tria", i32), ("qr_degree_quad", i32)]


class lfg_edge_mass_provider(C.Structure):
    _fields_ = [("gamma", lfg_coeff), ("edge_flags_dev", vp), ("qr_degree", i32)]


class lfg_edge_load_provider(C.Structure):
    _fields_ = [("g", lfg_coeff), ("edge_flags_dev", vp), ("qr_degree", i32)]


class lfg_solve_opts(C.Structure):
    _fields_ = [("precision", i32), ("max_iterations", i32), ("rtol", dbl), ("inner_rtol", dbl),
                ("check_every", i32)]


class lfg_solve_stats(C.Structure):
    _fields_ = [("iterations", i32), ("refinements", i32), ("rel_residual", dbl), ("converged", i32)]


class lfg_rd_adjoint_opts(C.Structure):
    _fields_ = [("load", lfg_load_provider), ("qr_degree_tria", i32), ("qr_degree_quad", i32),
                ("flags_dev", vp), ("dirichlet_dev", vp), ("solve", lfg_solve_opts), ("recompute", i32)]


class lfg_integrand(C.Structure):
    _fields_ = [("kind", i32), ("u", lfg_coeff), ("space", vp), ("dofs_dev", vp)]


# name -> (restype, argtypes)
SIGNATURES = {
    "lfg_ctx_create": (c_status, [C.c_int, P(vp)]),
    "lfg_ctx_destroy": (c_status, [vp]),
    "lfg_ctx_last_error": (C.c_char_p, [vp]),
    "lfg_ctx_stream": (vp, [vp]),
    "lfg_ctx_synchronize": (c_status, [vp]),
    "lfg_ctx_launch_count": (c_status, [vp, P(i64)]),
    "lfg_malloc": (c_status, [vp, sz, P(vp)]),
    "lfg_free": (c_status, [vp, vp]),
    "lfg_host_alloc": (c_status, [vp, sz, P(vp)]),
    "lfg_host_free": (c_status, [vp, vp]),
    "lfg_memcpy_h2d": (c_status, [vp, vp, vp, sz]),
    "lfg_memcpy_d2h": (c_status, [vp, vp, vp, sz]),
    "lfg_memcpy_d2d": (c_status, [vp, vp, vp, sz]),
    "lfg_memset": (c_status, [vp, vp, C.c_int, sz]),
    "lfg_timer_begin": (c_status, [vp]),
    "lfg_timer_end": (c_status, [vp, P(C.c_float)]),
    "lfg_l2_flush": (c_status, [vp]),
    "lfg_profile_enable": (c_status, [vp, C.c_int]),
    "lfg_profile_read": (c_status, [vp, C.c_char_p, P(dbl), P(i64)]),
    "lfg_profile_reset": (c_status, [vp]),
    "lfg_measure_fp64_peak": (c_status, [vp, P(dbl)]),
    "lfg_quad_rule": (c_status, [i32, i32, P(dbl), P(dbl), P(dbl), P(i32)]),
    "lfg_hier_dual": (c_status, [i32, i32, P(i32), i32, P(dbl), P(dbl), P(i32), P(i32)]),
    "lfg_ctx_set_tensor_cores": (c_status, [vp, i32]),
    "lfg_mesh_create": (c_status, [vp, i64, P(dbl), i64, P(i32), i64, P(i32), P(vp)]),
    "lfg_mesh_create_tp_triag": (c_status, [vp, i64, i64, dbl, dbl, dbl, dbl, P(vp)]),
    "lfg_mesh_create_tp_quad": (c_status, [vp, i64, i64, dbl, dbl, dbl, dbl, P(vp)]),
    "lfg_mesh_destroy": (c_status, [vp]),
    "lfg_mesh_sizes": (c_status, [vp, P(i64), P(i64), P(i64), P(i64), P(i64)]),
    "lfg_mesh_download_topology": (c_status, [vp, P(i32), P(i32), P(i8), P(i32)]),
    "lfg_mesh_device_arrays": (c_status, [vp, P(vp), P(vp)]),
    "lfg_mesh_set_coords": (c_status, [vp, vp, C.c_int]),
    "lfg_mesh_boundary_flags": (c_status, [vp, vp, vp]),
    "lfg_space_create": (c_status, [vp, C.c_int, C.c_int, C.c_int, C.c_int, P(vp)]),
    "lfg_space_create_lagrange": (c_status, [vp, C.c_int, P(vp)]),
    "lfg_space_create_hierarchic": (c_status, [vp, i32, P(vp)]),
    "lfg_space_create_hierarchic_var": (c_status, [vp, P(i32), P(i32), P(vp)]),
    "lfg_space_download_local_counts": (c_status, [vp, P(i32)]),
    "lfg_space_destroy": (c_status, [vp]),
    "lfg_space_info": (c_status, [vp, P(i64), P(i32), P(i32), P(i32), P(i64)]),
    "lfg_space_download_cell_dofs": (c_status, [vp, P(i32)]),
    "lfg_space_download_dof_entities": (c_status, [vp, P(i8), P(i32)]),
    "lfg_space_boundary_dof_flags": (c_status, [vp, vp]),
    "lfg_coo_create": (c_status, [vp, i64, i64, i64, P(vp)]),
    "lfg_coo_wrap": (c_status, [vp, i64, i64, vp, i64, i64, P(vp)]),
    "lfg_coo_destroy": (c_status, [vp]),
    "lfg_coo_size": (c_status, [vp, P(i64)]),
    "lfg_coo_triplets": (c_status, [vp, P(vp)]),
    "lfg_coo_set_zero": (c_status, [vp]),
    "lfg_coo_download": (c_status, [vp, vp, i64]),
    "lfg_coo_append_host": (c_status, [vp, vp, i64]),
    "lfg_assemble_matrix_rd": (c_status, [vp, P(lfg_rd_provider), vp]),
    "lfg_assemble_matrix_rd_to_host": (c_status, [vp, P(lfg_rd_provider), vp, i64, i64, P(i64)]),
    "lfg_assemble_vector_load": (c_status, [vp, P(lfg_load_provider), vp]),
    "lfg_assemble_matrix_edge_mass": (c_status, [vp, P(lfg_edge_mass_provider), vp]),
    "lfg_assemble_vector_edge_load": (c_status, [vp, P(lfg_edge_load_provider), vp]),
    "lfg_assemble_matrix_tabulated": (c_status, [vp, vp, i32, vp]),
    "lfg_assemble_vector_tabulated": (c_status, [vp, vp, i32, vp]),
    "lfg_fix_flagged_solution_components": (c_status, [vp, vp, vp, vp]),
    "lfg_fix_flagged_solution_comp_alt": (c_status, [vp, vp, vp, vp]),
    "lfg_fix_solution_components_lse": (c_status, [vp, i64, vp, vp, vp]),
    "lfg_csr_from_coo": (c_status, [vp, P(vp)]),
    "lfg_csr_destroy": (c_status, [vp]),
    "lfg_csr_info": (c_status, [vp, P(i64), P(i64), P(i64)]),
    "lfg_csr_download": (c_status, [vp, P(i64), P(i32), P(dbl)]),
    "lfg_csr_spmv": (c_status, [vp, vp, vp]),
    "lfg_solve_pcg": (c_status, [vp, vp, vp, P(lfg_solve_opts), P(lfg_solve_stats)]),
    "lfg_solve_pcg_noalloc": (c_status, [vp, vp, vp, P(lfg_solve_opts), P(lfg_solve_stats)]),
    "lfg_loss_l2_misfit": (c_status, [vp, i64, vp, vp, P(dbl), vp]),
    "lfg_grad_rd_cellwise": (c_status, [vp, P(lfg_rd_provider), vp, vp, vp, vp]),
    "lfg_rd_adjoint_create": (c_status, [vp, P(lfg_rd_adjoint_opts), vp, P(vp)]),
    "lfg_rd_adjoint_destroy": (c_status, [vp]),
    "lfg_rd_adjoint_forward": (c_status, [vp, vp, P(dbl), vp]),
    "lfg_rd_adjoint_backward": (c_status, [vp, dbl, vp]),
    "lfg_rd_adjoint_stats": (c_status, [vp, P(lfg_solve_stats), P(lfg_solve_stats), P(i64)]),
    "lfg_batch_create": (c_status, [vp, i32, P(vp), P(vp)]),
    "lfg_batch_destroy": (c_status, [vp]),
    "lfg_batch_info": (c_status, [vp, P(i32), P(i64), P(i64), P(i64)]),
    "lfg_batch_offsets": (c_status, [vp, P(i64), P(i64), P(i64)]),
    "lfg_batch_assemble_matrix_rd": (c_status, [vp, P(lfg_rd_provider), vp]),
    "lfg_batch_tuning": (c_status, [vp, P(i32), P(i32), P(dbl)]),
    "lfg_batch_assemble_vector_load": (c_status, [vp, P(lfg_load_provider), vp]),
    "lfg_batch_boundary_dof_flags": (c_status, [vp, vp]),
    "lfg_batch_solve_pcg": (c_status, [vp, vp, vp, vp, P(lfg_solve_opts), P(lfg_solve_stats), P(lfg_solve_stats)]),
    "lfg_batch_solve_tuning": (c_status, [vp, i32, P(i32), P(dbl)]),
    "lfg_batch_set_solve_chunk_rows": (c_status, [vp, i32, i32]),
    "lfg_batch_set_solve_groups": (c_status, [vp, dbl]),
    "lfg_batch_solve_groups": (c_status, [vp, P(dbl)]),
    "lfg_gmsh_last_error": (C.c_char_p, []),
    "lfg_gmsh_open": (c_status, [C.c_char_p, P(vp)]),
    "lfg_gmsh_open_buffer": (c_status, [C.c_char_p, i64, P(vp)]),
    "lfg_gmsh_destroy": (c_status, [vp]),
    "lfg_gmsh_sizes": (c_status, [vp, P(i64), P(i64), P(i64)]),
    "lfg_gmsh_factory_input": (c_status, [vp, P(dbl), P(i32), P(i32)]),
    "lfg_gmsh_build_mesh": (c_status, [vp, vp, P(vp)]),
    "lfg_gmsh_physical_entity_nrs": (c_status, [vp, i32, i64, P(i64), P(i32)]),
    "lfg_gmsh_is_physical_entity": (c_status, [vp, i32, i32, i64, P(u8)]),
    "lfg_gmsh_name_to_nr": (c_status, [vp, C.c_char_p, i32, P(i32)]),
    "lfg_gmsh_nr_to_name": (c_status, [vp, i32, i32, C.c_char_p, i64]),
    "lfg_gmsh_physical_entities": (c_status, [vp, i32, P(i32), P(i32)]),
    "lfg_integrate_mesh_function": (c_status, [vp, P(lfg_integrand), i32, vp, i32, P(dbl)]),
    "lfg_fe_eval": (c_status, [vp, vp, i32, P(dbl), vp, vp]),
    "lfg_nodal_projection": (c_status, [vp, P(lfg_coeff), vp, vp]),
    "lfg_init_essential_condition": (c_status, [vp, vp, P(lfg_coeff), vp, vp]),
}


def declare(lib):
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib
