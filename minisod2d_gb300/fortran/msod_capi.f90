! msod_capi.f90 -- ISO_C_BINDING interfaces of libmsod (include/msod.h) for a Fortran host.
!
! The reference driver (src/app/sources/main.f90) calls full_convec_ijk (elem_convec.f90:198),
! full_convec_ijk_split (:433), full_diffusion_ijk (elem_diffu.f90:10), fem_convec
! (elem_convec.f90:839) and fem_diffu (elem_diffu.f90:199) on device-resident arrays.  With this
! module in scope it calls msod_convec_ijk, msod_convec_ijk_split, msod_diffusion_ijk,
! msod_fem_convec and msod_fem_diffu instead, passing the device addresses of the same arrays
! (type(c_ptr): from msod_malloc, or c_loc inside "!$acc host_data use_device(...)") in the same
! layouts, with porder first and a CUDA stream (c_null_ptr: the default stream) last.  Every
! function returns MSOD_OK or an MSOD_ERR_* code; msod_last_error_string returns a C string.
!
! One interface per declaration of include/msod.h, in its order: scalars by value (C int ->
! integer(c_int), float -> real(c_float), double -> real(c_double), size_t -> integer(c_size_t),
! int64_t and uint64_t -> integer(c_int64_t)), pointers as type(c_ptr) by value, and the
! pointer-to-pointer outputs (msod_malloc, msod_mlp_create) as type(c_ptr) by reference.
! tests/test_fortran_module.py checks names, argument counts, kinds and attributes against the
! header, so the two cannot drift apart.
module msod_capi
   use iso_c_binding
   implicit none
   integer(c_int), parameter :: MSOD_VERSION = 100
   integer(c_int), parameter :: MSOD_MAX_PORDER = 8
   integer(c_int), parameter :: MSOD_OK = 0
   integer(c_int), parameter :: MSOD_ERR_INVALID_ARG = 1
   integer(c_int), parameter :: MSOD_ERR_PORDER = 2
   integer(c_int), parameter :: MSOD_ERR_CUDA = 3
   integer(c_int), parameter :: MSOD_ERR_BAD_TABLES = 4
   integer(c_int), parameter :: MSOD_ERR_NO_DEVICE = 5
   integer(c_int), parameter :: MSOD_ERR_INTERNAL = 6
   integer(c_int), parameter :: MSOD_ERR_UNSUPPORTED = 7
   integer(c_int), parameter :: MSOD_ERR_BAD_MODEL = 8
   integer(c_int), parameter :: MSOD_MLP_NFEATURES = 12
   integer(c_int), parameter :: MSOD_MLP_NPARAMS = 1505
   integer(c_int), parameter :: MSOD_FIELDS_SMOOTH = 0
   integer(c_int), parameter :: MSOD_FIELDS_SHOCK = 1
   integer(c_int), parameter :: MSOD_PREC_FP16 = 0
   integer(c_int), parameter :: MSOD_PREC_BF16 = 1
   integer(c_int), parameter :: MSOD_PREC_FP32 = 2
   integer(c_int), parameter :: MSOD_MU_E_GIVEN = 0
   integer(c_int), parameter :: MSOD_MU_E_PLAIN = 1
   integer(c_int), parameter :: MSOD_MU_E_LEARNED = 2
   interface
      integer(c_int) function msod_init(device) bind(C, name="msod_init")
         import :: c_int
         integer(c_int), value :: device
      end function msod_init
      integer(c_int) function msod_finalize() bind(C, name="msod_finalize")
         import :: c_int
      end function msod_finalize
      type(c_ptr) function msod_last_error_string() bind(C, name="msod_last_error_string")
         import :: c_ptr
      end function msod_last_error_string
      integer(c_int) function msod_version() bind(C, name="msod_version")
         import :: c_int
      end function msod_version
      integer(c_int) function msod_set_checked(enabled) bind(C, name="msod_set_checked")
         import :: c_int
         integer(c_int), value :: enabled
      end function msod_set_checked
      integer(c_int) function msod_malloc(ptr, bytes) bind(C, name="msod_malloc")
         import :: c_int, c_ptr, c_size_t
         type(c_ptr) :: ptr
         integer(c_size_t), value :: bytes
      end function msod_malloc
      integer(c_int) function msod_free(ptr) bind(C, name="msod_free")
         import :: c_int, c_ptr
         type(c_ptr), value :: ptr
      end function msod_free
      integer(c_int) function msod_h2d(dst_device, src_host, bytes, stream) bind(C, name="msod_h2d")
         import :: c_int, c_ptr, c_size_t
         type(c_ptr), value :: dst_device
         type(c_ptr), value :: src_host
         integer(c_size_t), value :: bytes
         type(c_ptr), value :: stream
      end function msod_h2d
      integer(c_int) function msod_d2h(dst_host, src_device, bytes, stream) bind(C, name="msod_d2h")
         import :: c_int, c_ptr, c_size_t
         type(c_ptr), value :: dst_host
         type(c_ptr), value :: src_device
         integer(c_size_t), value :: bytes
         type(c_ptr), value :: stream
      end function msod_d2h
      integer(c_int) function msod_memset(dst_device, value, bytes, stream) bind(C, name="msod_memset")
         import :: c_int, c_ptr, c_size_t
         type(c_ptr), value :: dst_device
         integer(c_int), value :: value
         integer(c_size_t), value :: bytes
         type(c_ptr), value :: stream
      end function msod_memset
      integer(c_int) function msod_stream_synchronize(stream) bind(C, name="msod_stream_synchronize")
         import :: c_int, c_ptr
         type(c_ptr), value :: stream
      end function msod_stream_synchronize
      integer(c_int) function msod_convec_ijk(porder, nelem, npoin, connec, Ngp, dNgp, He, gpvol, &
            dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, &
            Rener, stream) bind(C, name="msod_convec_ijk")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: xgp
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_convec_ijk
      integer(c_int) function msod_convec_ijk_split(porder, nelem, npoin, connec, Ngp, dNgp, He, &
            gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, &
            Rmass, Rmom, Rener, stream) bind(C, name="msod_convec_ijk_split")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: xgp
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_convec_ijk_split
      integer(c_int) function msod_diffusion_ijk(porder, nelem, npoin, connec, Ngp, dNgp, He, &
            gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, &
            mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_diffusion_ijk")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: xgp
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk

      integer(c_int) function msod_convec_diffusion_ijk(porder, nelem, npoin, connec, Ngp, dNgp, &
            He, gpvol, dlxigp_ip, xgp, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, u, q, rho, &
            press, E, Tem, mu_fluid, mu_e, mu_sgs, Rmass_c, Rmom_c, Rener_c, Rmass_d, Rmom_d, Rener_d, &
            stream) bind(C, name="msod_convec_diffusion_ijk")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: xgp
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: press
         type(c_ptr), value :: E
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass_c
         type(c_ptr), value :: Rmom_c
         type(c_ptr), value :: Rener_c
         type(c_ptr), value :: Rmass_d
         type(c_ptr), value :: Rmom_d
         type(c_ptr), value :: Rener_d
         type(c_ptr), value :: stream
      end function msod_convec_diffusion_ijk
      integer(c_int) function msod_convec_ijk_f64(porder, nelem, npoin, connec, He, gpvol, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, Rmass, Rmom, &
            Rener, stream) bind(C, name="msod_convec_ijk_f64")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_convec_ijk_f64
      integer(c_int) function msod_diffusion_ijk_f64(porder, nelem, npoin, connec, He, gpvol, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, &
            mu_e, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_diffusion_ijk_f64")
         import :: c_double, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_double), value :: Cp
         real(c_double), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk_f64
      integer(c_int) function msod_convec_ijk_mixed(precision, porder, nelem, npoin, connec, He, &
            gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, u, q, rho, pr, E, Rmass, &
            Rmom, Rener, stream) bind(C, name="msod_convec_ijk_mixed")
         import :: c_int, c_ptr
         integer(c_int), value :: precision
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_convec_ijk_mixed
      integer(c_int) function msod_diffusion_ijk_mixed(precision, porder, nelem, npoin, connec, He, &
            gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, &
            mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_diffusion_ijk_mixed")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: precision
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk_mixed
      integer(c_int) function msod_diffusion_ijk_mixed_nu(precision, porder, nelem, npoin, connec, &
            He, gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, &
            mu_fluid, nu_elem, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_diffusion_ijk_mixed_nu")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: precision
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk_mixed_nu
      integer(c_int) function msod_check_element_tables(porder, nelem, npoin, connec, dlxigp_ip, &
            invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, stream) bind(C, name="msod_check_element_tables")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: stream
      end function msod_check_element_tables
      integer(c_int) function msod_check_element_tables_noalloc(porder, nelem, npoin, connec, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, stream &
            ) bind(C, name="msod_check_element_tables_noalloc")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: stream
      end function msod_check_element_tables_noalloc
      integer(c_int) function msod_elem_jacobian(porder, nelem, npoin, connec, coord, dNgp, wgp, &
            gpvol, He, stream) bind(C, name="msod_elem_jacobian")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: He
         type(c_ptr), value :: stream
      end function msod_elem_jacobian
      integer(c_int) function msod_elem_jacobian_f64(porder, nelem, npoin, connec, coord, dNgp, &
            wgp, gpvol, He, stream) bind(C, name="msod_elem_jacobian_f64")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: He
         type(c_ptr), value :: stream
      end function msod_elem_jacobian_f64
      integer(c_int) function msod_fem_element_tables(porder, invAtoIJK, AtoIJK, AtoI, AtoJ, AtoK, &
            xgp, wgp, Ngp, dNgp, dlxigp_ip) bind(C, name="msod_fem_element_tables")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: AtoIJK
         type(c_ptr), value :: AtoI
         type(c_ptr), value :: AtoJ
         type(c_ptr), value :: AtoK
         type(c_ptr), value :: xgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: dlxigp_ip
      end function msod_fem_element_tables
      integer(c_int) function msod_fem_element_tables_f64(porder, invAtoIJK, AtoIJK, AtoI, AtoJ, &
            AtoK, xgp, wgp, Ngp, dNgp, dlxigp_ip) bind(C, name="msod_fem_element_tables_f64")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: AtoIJK
         type(c_ptr), value :: AtoI
         type(c_ptr), value :: AtoJ
         type(c_ptr), value :: AtoK
         type(c_ptr), value :: xgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: dlxigp_ip
      end function msod_fem_element_tables_f64
      integer(c_int) function msod_mesh_structured(porder, nx, ny, nz, AtoI, AtoJ, AtoK, jitter, &
            seed, connec, coord) bind(C, name="msod_mesh_structured")
         import :: c_double, c_int, c_int64_t, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nx
         integer(c_int), value :: ny
         integer(c_int), value :: nz
         type(c_ptr), value :: AtoI
         type(c_ptr), value :: AtoJ
         type(c_ptr), value :: AtoK
         real(c_double), value :: jitter
         integer(c_int64_t), value :: seed
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
      end function msod_mesh_structured
      integer(c_int) function msod_mesh_disconnected(porder, nelem, xyzBase, connec, coord &
            ) bind(C, name="msod_mesh_disconnected")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         type(c_ptr), value :: xyzBase
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
      end function msod_mesh_disconnected
      integer(c_int) function msod_reference_ic(porder, nelem, npoin, connec, u, q, rho, pr, E, &
            Tem, mu_fluid, mu_e, mu_sgs) bind(C, name="msod_reference_ic")
         import :: c_int, c_int64_t, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int64_t), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
      end function msod_reference_ic
      integer(c_int) function msod_fields_recipe(kind, nmodes, seed, npoin, coord, rho, u, q, pr, &
            E, Tem, mu_fluid) bind(C, name="msod_fields_recipe")
         import :: c_int, c_int64_t, c_ptr
         integer(c_int), value :: kind
         integer(c_int), value :: nmodes
         integer(c_int64_t), value :: seed
         integer(c_int64_t), value :: npoin
         type(c_ptr), value :: coord
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
      end function msod_fields_recipe
      integer(c_int) function msod_fem_convec(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, &
            rho, pr, E, Rmass, Rmom, Rener, stream) bind(C, name="msod_fem_convec")
         import :: c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_fem_convec
      integer(c_int) function msod_fem_convec_f64(nelem, npoin, connec, Ngp, dNgp, He, gpvol, u, q, &
            rho, pr, E, Rmass, Rmom, Rener, stream) bind(C, name="msod_fem_convec_f64")
         import :: c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: u
         type(c_ptr), value :: q
         type(c_ptr), value :: rho
         type(c_ptr), value :: pr
         type(c_ptr), value :: E
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_fem_convec_f64
      integer(c_int) function msod_fem_diffu(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, Pr, &
            rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_fem_diffu")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_fem_diffu
      integer(c_int) function msod_fem_diffu_f64(nelem, npoin, connec, Ngp, dNgp, He, gpvol, Cp, &
            Pr, rho, u, Tem, mu_fluid, mu_e, mu_sgs, Rmass, Rmom, Rener, stream &
            ) bind(C, name="msod_fem_diffu_f64")
         import :: c_double, c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         real(c_double), value :: Cp
         real(c_double), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_fem_diffu_f64
      integer(c_int) function msod_tet_jacobian(nelem, npoin, connec, coord, dNgp, wgp, gpvol, He, &
            stream) bind(C, name="msod_tet_jacobian")
         import :: c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: He
         type(c_ptr), value :: stream
      end function msod_tet_jacobian
      integer(c_int) function msod_tet_jacobian_f64(nelem, npoin, connec, coord, dNgp, wgp, gpvol, &
            He, stream) bind(C, name="msod_tet_jacobian_f64")
         import :: c_int, c_ptr
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: wgp
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: He
         type(c_ptr), value :: stream
      end function msod_tet_jacobian_f64
      integer(c_int) function msod_tet_element_tables(Ngp, dNgp, xgp, wgp &
            ) bind(C, name="msod_tet_element_tables")
         import :: c_int, c_ptr
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: xgp
         type(c_ptr), value :: wgp
      end function msod_tet_element_tables
      integer(c_int) function msod_tet_element_tables_f64(Ngp, dNgp, xgp, wgp &
            ) bind(C, name="msod_tet_element_tables_f64")
         import :: c_int, c_ptr
         type(c_ptr), value :: Ngp
         type(c_ptr), value :: dNgp
         type(c_ptr), value :: xgp
         type(c_ptr), value :: wgp
      end function msod_tet_element_tables_f64
      integer(c_int) function msod_tet_mesh_disconnected(nelem, xyzBase, connec, coord &
            ) bind(C, name="msod_tet_mesh_disconnected")
         import :: c_int, c_ptr
         integer(c_int), value :: nelem
         type(c_ptr), value :: xyzBase
         type(c_ptr), value :: connec
         type(c_ptr), value :: coord
      end function msod_tet_mesh_disconnected
      integer(c_int) function msod_entropy_viscosity(porder, nelem, npoin, connec, He, gpvol, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, rho, u, pr, gamma, ce, cmax, &
            normalise, mu_e, nu_elem, numax_elem, stream) bind(C, name="msod_entropy_viscosity")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: pr
         real(c_float), value :: gamma
         real(c_float), value :: ce
         real(c_float), value :: cmax
         integer(c_int), value :: normalise
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: numax_elem
         type(c_ptr), value :: stream
      end function msod_entropy_viscosity
      integer(c_int) function msod_mlp_features(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, &
            invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, rho, u, p_or_T, Rgas, gamma, cmax, feat, &
            numax_elem, stream) bind(C, name="msod_mlp_features")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: p_or_T
         real(c_float), value :: Rgas
         real(c_float), value :: gamma
         real(c_float), value :: cmax
         type(c_ptr), value :: feat
         type(c_ptr), value :: numax_elem
         type(c_ptr), value :: stream
      end function msod_mlp_features
      integer(c_int) function msod_mlp_create(out, seed) bind(C, name="msod_mlp_create")
         import :: c_int, c_int64_t, c_ptr
         type(c_ptr) :: out
         integer(c_int64_t), value :: seed
      end function msod_mlp_create
      integer(c_int) function msod_mlp_destroy(m) bind(C, name="msod_mlp_destroy")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
      end function msod_mlp_destroy
      integer(c_int) function msod_mlp_train(m, feat, target, weight, nsamples, steps, batch, lr, &
            seed, loss_host, stream) bind(C, name="msod_mlp_train")
         import :: c_float, c_int, c_int64_t, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: feat
         type(c_ptr), value :: target
         type(c_ptr), value :: weight
         integer(c_int), value :: nsamples
         integer(c_int), value :: steps
         integer(c_int), value :: batch
         real(c_float), value :: lr
         integer(c_int64_t), value :: seed
         type(c_ptr), value :: loss_host
         type(c_ptr), value :: stream
      end function msod_mlp_train
      integer(c_int) function msod_mlp_gradient(m, feat, target, weight, idx, batch, grad_host, &
            stream) bind(C, name="msod_mlp_gradient")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: feat
         type(c_ptr), value :: target
         type(c_ptr), value :: weight
         type(c_ptr), value :: idx
         integer(c_int), value :: batch
         type(c_ptr), value :: grad_host
         type(c_ptr), value :: stream
      end function msod_mlp_gradient
      integer(c_int) function msod_mlp_get_params(m, params_host, norm_host &
            ) bind(C, name="msod_mlp_get_params")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: params_host
         type(c_ptr), value :: norm_host
      end function msod_mlp_get_params
      integer(c_int) function msod_mlp_set_params(m, params_host, norm_host &
            ) bind(C, name="msod_mlp_set_params")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: params_host
         type(c_ptr), value :: norm_host
      end function msod_mlp_set_params
      integer(c_int) function msod_mlp_predict(m, feat, numax_elem, nelem, y, nu_elem, flag, stream &
            ) bind(C, name="msod_mlp_predict")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: feat
         type(c_ptr), value :: numax_elem
         integer(c_int), value :: nelem
         type(c_ptr), value :: y
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: flag
         type(c_ptr), value :: stream
      end function msod_mlp_predict
      integer(c_int) function msod_mlp_save(m, path) bind(C, name="msod_mlp_save")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: path
      end function msod_mlp_save
      integer(c_int) function msod_mlp_load(m, path) bind(C, name="msod_mlp_load")
         import :: c_int, c_ptr
         type(c_ptr), value :: m
         type(c_ptr), value :: path
      end function msod_mlp_load
      integer(c_int) function msod_learned_viscosity(m, porder, nelem, npoin, connec, He, gpvol, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, rho, u, p_or_T, Rgas, gamma, ce, &
            cmax, nu_elem, flag, stream) bind(C, name="msod_learned_viscosity")
         import :: c_float, c_int, c_ptr
         type(c_ptr), value :: m
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: p_or_T
         real(c_float), value :: Rgas
         real(c_float), value :: gamma
         real(c_float), value :: ce
         real(c_float), value :: cmax
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: flag
         type(c_ptr), value :: stream
      end function msod_learned_viscosity
      integer(c_int) function msod_diffusion_ijk_learned(m, porder, nelem, npoin, connec, He, &
            gpvol, dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, &
            mu_fluid, mu_sgs, p_or_T, Rgas, gamma, ce, cmax, Rmass, Rmom, Rener, nu_elem, flag, &
            stream) bind(C, name="msod_diffusion_ijk_learned")
         import :: c_float, c_int, c_ptr
         type(c_ptr), value :: m
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: p_or_T
         real(c_float), value :: Rgas
         real(c_float), value :: gamma
         real(c_float), value :: ce
         real(c_float), value :: cmax
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: flag
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk_learned
      integer(c_int) function msod_diffusion_ijk_nu(porder, nelem, npoin, connec, He, gpvol, &
            dlxigp_ip, invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, rho, u, Tem, mu_fluid, &
            nu_elem, mu_sgs, Rmass, Rmom, Rener, stream) bind(C, name="msod_diffusion_ijk_nu")
         import :: c_float, c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         type(c_ptr), value :: rho
         type(c_ptr), value :: u
         type(c_ptr), value :: Tem
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: nu_elem
         type(c_ptr), value :: mu_sgs
         type(c_ptr), value :: Rmass
         type(c_ptr), value :: Rmom
         type(c_ptr), value :: Rener
         type(c_ptr), value :: stream
      end function msod_diffusion_ijk_nu
      integer(c_int) function msod_set_mode(precision, mu_e_mode, mlp) bind(C, name="msod_set_mode")
         import :: c_int, c_ptr
         integer(c_int), value :: precision
         integer(c_int), value :: mu_e_mode
         type(c_ptr), value :: mlp
      end function msod_set_mode
      integer(c_int) function msod_get_mode(precision, mu_e_mode) bind(C, name="msod_get_mode")
         import :: c_int, c_ptr
         type(c_ptr), value :: precision
         type(c_ptr), value :: mu_e_mode
      end function msod_get_mode
      integer(c_int) function msod_lumped_mass(porder, nelem, npoin, connec, gpvol, Ml, &
            stream) bind(C, name="msod_lumped_mass")
         import :: c_int, c_ptr
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: Ml
         type(c_ptr), value :: stream
      end function msod_lumped_mass
      integer(c_int) function msod_rk4_workspace_bytes(npoin, bytes) bind(C, name="msod_rk4_workspace_bytes")
         import :: c_int, c_ptr
         integer(c_int), value :: npoin
         type(c_ptr), value :: bytes
      end function msod_rk4_workspace_bytes
      integer(c_int) function msod_rk4_step(porder, nelem, npoin, connec, He, gpvol, dlxigp_ip, &
            invAtoIJK, gmshAtoI, gmshAtoJ, gmshAtoK, Cp, Pr, gamma, Rgas, Ml, mu_fluid, mu_e, mu_sgs, &
            dt, rho, q, rhoE, workspace, workspace_bytes, stream) bind(C, name="msod_rk4_step")
         import :: c_int, c_ptr, c_float, c_size_t
         integer(c_int), value :: porder
         integer(c_int), value :: nelem
         integer(c_int), value :: npoin
         type(c_ptr), value :: connec
         type(c_ptr), value :: He
         type(c_ptr), value :: gpvol
         type(c_ptr), value :: dlxigp_ip
         type(c_ptr), value :: invAtoIJK
         type(c_ptr), value :: gmshAtoI
         type(c_ptr), value :: gmshAtoJ
         type(c_ptr), value :: gmshAtoK
         real(c_float), value :: Cp
         real(c_float), value :: Pr
         real(c_float), value :: gamma
         real(c_float), value :: Rgas
         type(c_ptr), value :: Ml
         type(c_ptr), value :: mu_fluid
         type(c_ptr), value :: mu_e
         type(c_ptr), value :: mu_sgs
         real(c_float), value :: dt
         type(c_ptr), value :: rho
         type(c_ptr), value :: q
         type(c_ptr), value :: rhoE
         type(c_ptr), value :: workspace
         integer(c_size_t), value :: workspace_bytes
         type(c_ptr), value :: stream
      end function msod_rk4_step
   end interface
end module msod_capi
