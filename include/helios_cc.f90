! helios_cc.f90 -- Fortran interface (iso_c_binding) to the C ABI of include/helios_cc.h.
!
! The GB300 closed-shell PPP CCSD engine is called from helios's Fortran host
! through this module: the derived types mirror hx_ppp_model and hx_cc_params
! field by field, and every entry point of helios_cc.h has an interface here
! with the same name. A helios build links libhelios_gb300.so and, in the
! routines that drive r-ccsd (getEnergy, src/modules/mod_property.f90:55-338),
! replaces setCCParameters / initCC / iterator / energyCC / finalizeCC
! (src/methods/coupledCluster/mod_cc.f90) by hx_ccsd_create / hx_ccsd_init /
! hx_ccsd_solve / hx_ccsd_energy / hx_ccsd_destroy; the adapter module a
! maintainer adds on top of this one (it reads helios's mol, ccbd and scfbd
! blocks) is listed in INTEGRATION.md.
!
! Conventions (as in the C header): every function returns 0 or a negative
! code; iteration statuses are 1 converged, -1 failed, -2 diverged,
! -3 stagnated, -4 interrupted; errors are <= -100 and hx_last_error gives
! the message. Amplitudes cross in helios's column-major layout t1(o, v),
! t2(o, o, v, v). Energies in eV, coordinates in Angstrom, fields in eV/A.
module helios_cc
    use iso_c_binding
    implicit none
    private

    integer(c_int), parameter, public :: HX_OK = 0, HX_CONVERGED = 1, HX_FAILED_MAXITER = -1, &
        HX_DIVERGED = -2, HX_STAGNATED = -3, HX_INTERRUPTED = -4, HX_ERR_ARG = -100, HX_ERR_CUDA = -101, &
        HX_ERR_NOMEM = -102, HX_ERR_STATE = -103, HX_ERR_SCF = -104, HX_ERR_KERNEL = -105, &
        HX_ERR_UNSUPPORTED = -106
    integer(c_int32_t), parameter, public :: HX_COULOMB_OHNO_KLOPMAN = 0, HX_COULOMB_MATAGA_NISHIMOTO = 1, &
        HX_COULOMB_HUBBARD = 2, HX_BOND_SINGLE = 0, HX_BOND_DOUBLE = 1, HX_BOND_NONSET = -1, &
        HX_PRECISION_FP64 = 0, HX_PRECISION_MIXED = 1, HX_PRECISION_EXACT = 2, &
        HX_NOALLOC_MAX_DIM = 512

    ! one molecule block (readMoleculeInformation.f90:20-117); pointers to arrays
    ! the caller keeps alive: coords(3, n_sites), alpha, gamma, nels (n_sites),
    ! bond_i, bond_j (0-based sites), beta, bond_kind (n_bonds)
    type, bind(c), public :: hx_ppp_model
        integer(c_int32_t) :: n_sites
        type(c_ptr)        :: coords, alpha, gamma, nels
        integer(c_int32_t) :: n_bonds
        type(c_ptr)        :: bond_i, bond_j, beta, bond_kind
    end type

    ! the keywords of the path (definebd.f90); hx_cc_params_default fills helios's defaults
    type, bind(c), public :: hx_cc_params
        integer(c_int32_t) :: coulomb
        real(c_double)     :: bond_alternation, field(3)
        integer(c_int32_t) :: scf_maxiter
        real(c_double)     :: scf_eps, scf_step
        integer(c_int32_t) :: projection_type, cc_maxiter
        real(c_double)     :: cc_eps, t1_step, t2_step
        integer(c_int32_t) :: diis_enabled, diis_steps, check_divergence
        real(c_double)     :: divergence_threshold
        integer(c_int32_t) :: check_stagnation
        real(c_double)     :: stagnation_threshold
        integer(c_int32_t) :: stagnation_after, precision, guess
        real(c_double)     :: mixed_switch
        integer(c_int32_t) :: mixed_patience, mixed_check, tile_tuning, tile_force
    end type

    public :: hx_cc_params_default, hx_ccsd_create, hx_ccsd_create_batch, hx_ccsd_init, hx_ccsd_set_guess
    public :: hx_mlp_nparam, hx_ccsd_set_model, hx_ccsd_training_rows, hx_mlp_predict, hx_mlp_grad, hx_mlp_train
    public :: hx_ccsd_iterate, hx_ccsd_energy, hx_ccsd_solve, hx_ccsd_solve_batch, hx_ccsd_get_amplitudes
    public :: hx_ccsd_get_scf, hx_ccsd_trace, hx_ccsd_triples, hx_ccsd_timing, hx_ccsd_dims, hx_ccsd_cancel
    public :: hx_ccsd_destroy, hx_gemm, hx_gemm_tile, hx_gemm_noalloc, hx_tile_table, hx_tile_table_load, hx_tile_variants
    public :: hx_ccsd_tile_choices, hx_last_error

    interface
        subroutine hx_cc_params_default(p) bind(c, name='hx_cc_params_default')
            import :: hx_cc_params
            type(hx_cc_params), intent(out) :: p
        end subroutine

        integer(c_int) function hx_ccsd_create(m, p, h) bind(c, name='hx_ccsd_create')
            import :: hx_ppp_model, hx_cc_params, c_ptr, c_int
            type(hx_ppp_model), intent(in) :: m
            type(hx_cc_params), intent(in) :: p
            type(c_ptr), intent(out) :: h
        end function

        integer(c_int) function hx_ccsd_create_batch(ms, n, p, h) bind(c, name='hx_ccsd_create_batch')
            import :: hx_ppp_model, hx_cc_params, c_ptr, c_int, c_int32_t
            type(hx_ppp_model), intent(in) :: ms(*)
            integer(c_int32_t), value :: n
            type(hx_cc_params), intent(in) :: p
            type(c_ptr), intent(out) :: h
        end function

        integer(c_int) function hx_ccsd_init(h) bind(c, name='hx_ccsd_init')
            import :: c_ptr, c_int
            type(c_ptr), value :: h
        end function

        integer(c_int) function hx_ccsd_set_guess(h, mol, t1, t2) bind(c, name='hx_ccsd_set_guess')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol
            real(c_double), intent(in) :: t1(*), t2(*)
        end function

        integer(c_int) function hx_mlp_nparam() bind(c, name='hx_mlp_nparam')
            import :: c_int
        end function

        integer(c_int) function hx_ccsd_set_model(h, params) bind(c, name='hx_ccsd_set_model')
            import :: c_ptr, c_int, c_float
            type(c_ptr), value :: h
            real(c_float), intent(in) :: params(*)
        end function

        integer(c_int) function hx_ccsd_training_rows(h, mol, n, rows, x, t) bind(c, name='hx_ccsd_training_rows')
            import :: c_ptr, c_int, c_int32_t, c_int64_t, c_float
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol, n
            integer(c_int64_t), intent(in) :: rows(*)
            real(c_float), intent(out) :: x(*), t(*)
        end function

        integer(c_int) function hx_mlp_predict(params, x, n, y) bind(c, name='hx_mlp_predict')
            import :: c_int, c_int64_t, c_float
            real(c_float), intent(in) :: params(*), x(*)
            integer(c_int64_t), value :: n
            real(c_float), intent(out) :: y(*)
        end function

        integer(c_int) function hx_mlp_grad(params, x, t, n, loss, grad) bind(c, name='hx_mlp_grad')
            import :: c_int, c_int32_t, c_float
            real(c_float), intent(in) :: params(*), x(*), t(*)
            integer(c_int32_t), value :: n
            real(c_float), intent(out) :: loss, grad(*)
        end function

        integer(c_int) function hx_mlp_train(params, x, t, n, epochs, batch, lr, seed, epoch_loss) &
                bind(c, name='hx_mlp_train')
            import :: c_int, c_int32_t, c_int64_t, c_float
            real(c_float), intent(inout) :: params(*)
            real(c_float), intent(in) :: x(*), t(*)
            integer(c_int64_t), value :: n, seed
            integer(c_int32_t), value :: epochs, batch
            real(c_float), value :: lr
            real(c_float), intent(out) :: epoch_loss(*)
        end function

        integer(c_int) function hx_ccsd_iterate(h, iteration, eps, acc) bind(c, name='hx_ccsd_iterate')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: iteration
            real(c_double), value :: eps
            real(c_double), intent(out) :: acc(5)
        end function

        integer(c_int) function hx_ccsd_energy(h, e) bind(c, name='hx_ccsd_energy')
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: e(5)
        end function

        integer(c_int) function hx_ccsd_solve(h, maxiter, eps, status, iters, e) bind(c, name='hx_ccsd_solve')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: maxiter
            real(c_double), value :: eps
            integer(c_int32_t), intent(out) :: status, iters
            real(c_double), intent(out) :: e(5)
        end function

        integer(c_int) function hx_ccsd_solve_batch(h, status, iters, e) bind(c, name='hx_ccsd_solve_batch')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), intent(out) :: status(*), iters(*)
            real(c_double), intent(out) :: e(5, *)
        end function

        integer(c_int) function hx_ccsd_get_amplitudes(h, mol, t1, t2) bind(c, name='hx_ccsd_get_amplitudes')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol
            real(c_double), intent(out) :: t1(*), t2(*)
        end function

        integer(c_int) function hx_ccsd_get_scf(h, mol, c, eps, fmo, scf, scf_status) bind(c, name='hx_ccsd_get_scf')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol
            real(c_double), intent(out) :: c(*), eps(*), fmo(*), scf(4)
            integer(c_int32_t), intent(out) :: scf_status(2)
        end function

        integer(c_int) function hx_ccsd_trace(h, mol, out, cap) bind(c, name='hx_ccsd_trace')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol, cap
            real(c_double), intent(out) :: out(5, *)
        end function

        integer(c_int) function hx_ccsd_triples(h, mol, e) bind(c, name='hx_ccsd_triples')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol
            real(c_double), intent(out) :: e(4)
        end function

        integer(c_int) function hx_ccsd_timing(h, out, profile) bind(c, name='hx_ccsd_timing')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            real(c_double), intent(out) :: out(8)
            integer(c_int32_t), value :: profile
        end function

        integer(c_int) function hx_ccsd_dims(h, mol, dims) bind(c, name='hx_ccsd_dims')
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value :: h
            integer(c_int32_t), value :: mol
            integer(c_int32_t), intent(out) :: dims(4)
        end function

        subroutine hx_ccsd_cancel(h) bind(c, name='hx_ccsd_cancel')
            import :: c_ptr
            type(c_ptr), value :: h
        end subroutine

        subroutine hx_ccsd_destroy(h) bind(c, name='hx_ccsd_destroy')
            import :: c_ptr
            type(c_ptr), value :: h
        end subroutine

        integer(c_int) function hx_gemm(a, b, c, m, n, k, precision, reps, ms) bind(c, name='hx_gemm')
            import :: c_int, c_int32_t, c_double
            real(c_double), intent(in) :: a(*), b(*)
            real(c_double), intent(out) :: c(*)
            integer(c_int32_t), value :: m, n, k, precision, reps
            real(c_double), intent(out) :: ms
        end function

        integer(c_int) function hx_gemm_tile(a, b, c, m, n, k, precision, variant, reps, ms) bind(c, name='hx_gemm_tile')
            import :: c_int, c_int32_t, c_double
            real(c_double), intent(in) :: a(*), b(*)
            real(c_double), intent(out) :: c(*)
            integer(c_int32_t), value :: m, n, k, precision, variant, reps
            real(c_double), intent(out) :: ms
        end function

        ! a, b, c are device addresses; stream is a cudaStream_t (c_null_ptr: the legacy default stream)
        integer(c_int) function hx_gemm_noalloc(a, b, c, m, n, k, precision, stream) bind(c, name='hx_gemm_noalloc')
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value :: a, b, c, stream
            integer(c_int32_t), value :: m, n, k, precision
        end function

        integer(c_int) function hx_tile_table(entries, cap) bind(c, name='hx_tile_table')
            import :: c_int, c_int32_t
            integer(c_int32_t), intent(out) :: entries(5, *)
            integer(c_int32_t), value :: cap
        end function

        integer(c_int) function hx_tile_table_load(entries, n) bind(c, name='hx_tile_table_load')
            import :: c_int, c_int32_t
            integer(c_int32_t), intent(in) :: entries(5, *)
            integer(c_int32_t), value :: n
        end function

        integer(c_int) function hx_tile_variants(mode, bn, cap) bind(c, name='hx_tile_variants')
            import :: c_int, c_int32_t
            integer(c_int32_t), value :: mode, cap
            integer(c_int32_t), intent(out) :: bn(*)
        end function

        integer(c_int) function hx_ccsd_tile_choices(h, var, cap, tune_ms) bind(c, name='hx_ccsd_tile_choices')
            import :: c_ptr, c_int, c_int32_t, c_double
            type(c_ptr), value :: h
            integer(c_int32_t), intent(out) :: var(*)
            integer(c_int32_t), value :: cap
            real(c_double), intent(out) :: tune_ms
        end function

        integer(c_int) function hx_last_error(buf, len) bind(c, name='hx_last_error')
            import :: c_int, c_char, c_size_t
            character(kind=c_char), intent(out) :: buf(*)
            integer(c_size_t), value :: len
        end function
    end interface
end module helios_cc
