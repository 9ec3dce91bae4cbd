! r-ccsd of all-trans dodecahexaene through the Fortran interface (include/helios_cc.f90):
! the calls a helios build makes, on the molecule helios's own examples run. Prints
! "status iterations E_total E_ref" for the test that compiles it.
program dodecahexaene
    use iso_c_binding
    use helios_cc
    implicit none
    integer, parameter :: n = 12
    real(c_double), target :: xyz(3, n), alp(n), gam(n), bet(n - 1)
    integer(c_int32_t), target :: ne(n), bi(n - 1), bj(n - 1), bk(n - 1)
    type(hx_ppp_model) :: m
    type(hx_cc_params) :: p
    type(c_ptr) :: h
    integer(c_int32_t) :: st, it
    real(c_double) :: e(5), r, ang
    integer :: k, rc
    real(c_double), parameter :: pi = 3.14159265358979323846d0

    xyz = 0d0
    do k = 1, n - 1                       ! zigzag chain: bonds 1.35 (double) / 1.46 (single), 120 degrees
        if (mod(k, 2) == 1) then
            r = 1.35d0; ang = 30d0; bk(k) = HX_BOND_DOUBLE
        else
            r = 1.46d0; ang = -30d0; bk(k) = HX_BOND_SINGLE
        end if
        xyz(1, k + 1) = xyz(1, k) + r * cos(ang * pi / 180d0)
        xyz(2, k + 1) = xyz(2, k) + r * sin(ang * pi / 180d0)
        bi(k) = k - 1; bj(k) = k; bet(k) = -2.4d0
    end do
    alp = 0d0; gam = 11.13d0; ne = 1
    m = hx_ppp_model(n, c_loc(xyz), c_loc(alp), c_loc(gam), c_loc(ne), n - 1, c_loc(bi), c_loc(bj), &
                     c_loc(bet), c_loc(bk))
    call hx_cc_params_default(p)
    p%bond_alternation = 0.1d0
    p%cc_eps = 1d-10
    rc = hx_ccsd_create(m, p, h)
    if (rc /= HX_OK) stop 1
    rc = hx_ccsd_init(h)
    if (rc /= HX_OK) stop 2
    rc = hx_ccsd_solve(h, p%cc_maxiter, p%cc_eps, st, it, e)
    if (rc /= HX_OK) stop 3
    write (*, '(i3, 1x, i5, 2(1x, es24.16))') st, it, e(1), e(2)
    call hx_ccsd_destroy(h)
end program dodecahexaene
