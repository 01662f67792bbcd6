! fempar_gpu.f90 -- ISO_C_BINDING interfaces of libfempar_gpu.so (include/fempar_gpu.h)
! for FEMPAR's Fortran drivers.  The derived types mirror the header's structs field for
! field; every function returns the library's fg_status (0 = FG_OK).  Source only: this
! image has no Fortran compiler, so tests/test_fortran_binding_doc.py checks the types
! against the C header textually.
module fempar_gpu_names
  use iso_c_binding
  implicit none
  integer(c_int32_t), parameter :: FG_OK = 0, FG_ERR_NOT_CONVERGED = -4
  integer(c_int), parameter :: FG_POISSON = 0, FG_ELASTICITY = 1
  integer(c_int), parameter :: FG_FN_ZERO = 0, FG_FN_CONST = 1, FG_FN_SHARP_WAVE = 2, FG_FN_LINEAR = 3, FG_FN_QP_VALUES = 4
  integer(c_int), parameter :: FG_PREC_NONE = 0, FG_PREC_JACOBI = 1, FG_FP64 = 0, FG_MIXED = 1
  integer(c_int), parameter :: FG_RES_RES = 0, FG_RES_RHS = 1, FG_DELTA_RHS = 2, FG_DELTA_DELTA = 3, &
                               FG_RES_NRMGIVEN_RHS_NRMGIVEN = 4, FG_RES_NRMGIVEN_RES_NRMGIVEN = 5

  type, bind(c) :: fg_integrand
    integer(c_int)  :: kind
    type(c_ptr)     :: cell_coef
    real(c_double)  :: coef_const, nu
    integer(c_int)  :: source_fn
    real(c_double)  :: fn_param(8)
    type(c_ptr)     :: qp_source
    integer(c_int)  :: boundary_fn
    type(c_ptr)     :: dirichlet_values
    integer(c_int)  :: flags
  end type

  type, bind(c) :: fg_solver_params
    integer(c_int) :: precond, precision, criterion
    real(c_double) :: rtol, atol
    integer(c_int) :: max_iters
    real(c_double) :: inner_rtol
    integer(c_int) :: inner_max_iters, check_every
  end type

  type, bind(c) :: fg_solve_info
    integer(c_int)     :: iterations, outer_iterations, converged
    real(c_double)     :: error_estimate, tolerance, solve_ms
    integer(c_int64_t) :: kernel_launches
  end type


  type, bind(c) :: fg_bddc_params
    integer(c_int32_t) :: nsub(3)
    type(c_ptr)        :: cuts            ! nsub(1)+1 + nsub(2)+1 + nsub(3)+1 cell indices, or c_null_ptr
    integer(c_int32_t) :: use_vertices, use_edges, use_faces, weighting
    integer(c_int32_t) :: coarse_handler  ! 0 standard, 1 elasticity (rigid-body face functionals)
    integer(c_int32_t) :: use_subparts    ! 1: physics-based partition (subparts of equal coefficient)
  end type

  type, bind(c) :: fg_error_norms
    real(c_double) :: mean_norm, l1_norm, l2_norm, linfty_norm
    real(c_double) :: h1_seminorm, h1_norm, w1infty_seminorm, w1infty_norm, energy_norm
  end type

  interface
    function fg_ctx_create(device, budget, ctx) bind(c, name="fg_ctx_create")
      import; integer(c_int32_t) :: fg_ctx_create
      integer(c_int), value :: device; integer(c_int64_t), value :: budget; type(c_ptr) :: ctx
    end function
    function fg_mesh_create_structured(ctx, num_dims, n, limits, vertex_xyz, mesh) bind(c, name="fg_mesh_create_structured")
      import; integer(c_int32_t) :: fg_mesh_create_structured
      type(c_ptr), value :: ctx; integer(c_int), value :: num_dims
      integer(c_int32_t) :: n(3); real(c_double) :: limits(6); type(c_ptr), value :: vertex_xyz; type(c_ptr) :: mesh
    end function
    function fg_space_create(mesh, order, ncomp, ids, n_ids, space) bind(c, name="fg_space_create")
      import; integer(c_int32_t) :: fg_space_create
      type(c_ptr), value :: mesh; integer(c_int), value :: order, ncomp, n_ids
      integer(c_int32_t) :: ids(*); type(c_ptr) :: space
    end function
    function fg_space_get_dof_map(space, lst_dofs_gids) bind(c, name="fg_space_get_dof_map")
      import; integer(c_int32_t) :: fg_space_get_dof_map
      type(c_ptr), value :: space; integer(c_int32_t) :: lst_dofs_gids(*)
    end function
    function fg_assemble(space, integrand, sys) bind(c, name="fg_assemble")
      import; integer(c_int32_t) :: fg_assemble
      type(c_ptr), value :: space; type(fg_integrand) :: integrand; type(c_ptr) :: sys
    end function
    function fg_system_reassemble(sys, integrand) bind(c, name="fg_system_reassemble")
      import; integer(c_int32_t) :: fg_system_reassemble
      type(c_ptr), value :: sys; type(fg_integrand) :: integrand
    end function
    function fg_system_export_csr(sys, symmetric_storage, one_based, irp, ja, val) bind(c, name="fg_system_export_csr")
      import; integer(c_int32_t) :: fg_system_export_csr
      type(c_ptr), value :: sys; integer(c_int), value :: symmetric_storage, one_based
      integer(c_int64_t) :: irp(*); integer(c_int32_t) :: ja(*); real(c_double) :: val(*)
    end function
    function fg_system_export_rhs(sys, rhs) bind(c, name="fg_system_export_rhs")
      import; integer(c_int32_t) :: fg_system_export_rhs
      type(c_ptr), value :: sys; real(c_double) :: rhs(*)
    end function
    function fg_solve(sys, params, b, x0, x, info) bind(c, name="fg_solve")
      import; integer(c_int32_t) :: fg_solve
      type(c_ptr), value :: sys; type(fg_solver_params) :: params
      type(c_ptr), value :: b, x0; real(c_double) :: x(*); type(fg_solve_info) :: info
    end function
    function fg_bddc_create(sys, params, bddc) bind(c, name="fg_bddc_create")
      import; integer(c_int32_t) :: fg_bddc_create
      type(c_ptr), value :: sys; type(fg_bddc_params) :: params; type(c_ptr) :: bddc
    end function
    function fg_bddc_numerical_setup(bddc) bind(c, name="fg_bddc_numerical_setup")
      import; integer(c_int32_t) :: fg_bddc_numerical_setup; type(c_ptr), value :: bddc
    end function
    function fg_bddc_solve(bddc, params, b, x0, x, info) bind(c, name="fg_bddc_solve")
      import; integer(c_int32_t) :: fg_bddc_solve
      type(c_ptr), value :: bddc; type(fg_solver_params) :: params
      type(c_ptr), value :: b, x0; real(c_double) :: x(*); type(fg_solve_info) :: info
    end function
    function fg_bddc_destroy(bddc) bind(c, name="fg_bddc_destroy")
      import; integer(c_int32_t) :: fg_bddc_destroy; type(c_ptr), value :: bddc
    end function
    function fg_system_error_norms(sys, x, x_on_device, fn, fn_param, cell_sq_energy, norms) &
        bind(c, name="fg_system_error_norms")
      import; integer(c_int32_t) :: fg_system_error_norms
      type(c_ptr), value :: sys, x, cell_sq_energy; integer(c_int32_t), value :: x_on_device, fn
      real(c_double) :: fn_param(8); type(fg_error_norms) :: norms
    end function
    function fg_mesh_read_gid(ctx, dir_path, prefix, mesh) bind(c, name="fg_mesh_read_gid")
      import; integer(c_int32_t) :: fg_mesh_read_gid
      type(c_ptr), value :: ctx
      character(kind=c_char) :: dir_path(*), prefix(*)      ! NUL-terminated
      type(c_ptr) :: mesh
    end function
    function fg_mesh_create_unstructured(ctx, num_vertices, vertex_xyz, num_cells, cell_vertices, &
        num_given_vefs, given_vef_ptr, given_vef_vertices, given_vef_set, mesh) &
        bind(c, name="fg_mesh_create_unstructured")
      import; integer(c_int32_t) :: fg_mesh_create_unstructured
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: num_vertices, num_cells, num_given_vefs
      real(c_double) :: vertex_xyz(3, *)                  ! mesh%coord
      integer(c_int32_t) :: cell_vertices(8, *)           ! mesh%lnods (z order), 1-based
      integer(c_int64_t) :: given_vef_ptr(*)              ! 0-based offsets of mesh%given_vefs
      integer(c_int32_t) :: given_vef_vertices(*), given_vef_set(*)
      type(c_ptr) :: mesh
    end function
    function fg_space_create_dg(mesh, order, space) bind(c, name="fg_space_create_dg")
      import; integer(c_int32_t) :: fg_space_create_dg
      type(c_ptr), value :: mesh; integer(c_int), value :: order; type(c_ptr) :: space
    end function
    function fg_partition_create(space, num_parts_x_dir, partition) bind(c, name="fg_partition_create")
      import; integer(c_int32_t) :: fg_partition_create
      type(c_ptr), value :: space; integer(c_int32_t) :: num_parts_x_dir(3); type(c_ptr) :: partition
    end function
    function fg_partition_comm_device(partition, x) bind(c, name="fg_partition_comm_device")
      import; integer(c_int32_t) :: fg_partition_comm_device
      type(c_ptr), value :: partition, x
    end function
    function fg_space_get_qp_coords(space, xyz, on_device) bind(c, name="fg_space_get_qp_coords")
      import; integer(c_int32_t) :: fg_space_get_qp_coords
      type(c_ptr), value :: space; real(c_double) :: xyz(3, *); integer(c_int), value :: on_device
    end function
    function fg_system_spmv_device_noalloc(sys, precision, x, y) bind(c, name="fg_system_spmv_device_noalloc")
      import; integer(c_int32_t) :: fg_system_spmv_device_noalloc
      type(c_ptr), value :: sys, x, y; integer(c_int), value :: precision
    end function
    ! C = alpha A B^T + beta C on device arrays, FP64 emulated on the tensor cores; A(i,l) at
    ! A[i*a_rs + l*a_cs] (column-major: a_rs = 1, a_cs = lda); b = c_null_ptr: B = A
    function fg_dense_gemm_nt(ctx, m, n, k, alpha, a, a_rs, a_cs, b, b_rs, b_cs, beta, c, c_rs, c_cs, flags) &
        bind(c, name="fg_dense_gemm_nt")
      import; integer(c_int32_t) :: fg_dense_gemm_nt
      type(c_ptr), value :: ctx, a, b, c
      integer(c_int64_t), value :: m, n, k, a_rs, a_cs, b_rs, b_cs, c_rs, c_cs
      real(c_double), value :: alpha, beta; integer(c_int32_t), value :: flags
    end function
  end interface
end module fempar_gpu_names
