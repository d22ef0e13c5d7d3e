! bs2e_gpu.f90 -- ISO_C_BINDING interface to libbs2e.so for basis_setup.
!
! The reference builds with -fdefault-integer-8 (CMakeLists.txt:45-53), so
! every integer crossing the boundary is integer(c_int64_t), and type(config)
! (src/tools/orbital_tools.f90:15-19) is passed as the bind(C) record
! bs2e_config_c.  Complex matrices are complex(c_double_complex), column-major,
! exactly the arrays basis_setup already holds (S, H_vec(l)%data).
module bs2e_gpu
    use iso_c_binding
    implicit none

    integer(c_int32_t), parameter :: BS2E_OK = 0
    integer(c_int64_t), parameter :: BS2E_PREC_FP64 = 0, BS2E_PREC_MIXED = 1

    type, bind(C) :: bs2e_config_c
        integer(c_int64_t) :: n1, n2, l1, l2, eqv
    end type bs2e_config_c

    type, bind(C) :: bs2e_opts_c
        integer(c_int64_t) :: precision, device
        integer(c_int64_t) :: stage_bytes    ! HBM staging per area for host-array fills (0 = 8 GiB)
        integer(c_int64_t) :: reserved(5)
    end type bs2e_opts_c

    interface
        subroutine bs2e_default_opts(opts) bind(C, name="bs2e_default_opts")
            import :: bs2e_opts_c
            type(bs2e_opts_c), intent(out) :: opts
        end subroutine

        integer(c_int32_t) function bs2e_create(knots, n_knots, k, k_GL, max_k, opts, h) &
                bind(C, name="bs2e_create")
            import :: c_int32_t, c_int64_t, c_double, c_ptr, bs2e_opts_c
            real(c_double), intent(in) :: knots(*)
            integer(c_int64_t), value :: n_knots, k, k_GL, max_k
            type(bs2e_opts_c), intent(in) :: opts
            type(c_ptr), intent(out) :: h
        end function

        integer(c_int32_t) function bs2e_destroy(h) bind(C, name="bs2e_destroy")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int32_t) function bs2e_last_error(h, buf, buflen) bind(C, name="bs2e_last_error")
            import :: c_int32_t, c_int64_t, c_ptr, c_char
            type(c_ptr), value :: h
            character(kind=c_char), intent(out) :: buf(*)
            integer(c_int64_t), value :: buflen
        end function

        integer(c_int32_t) function bs2e_slater(h) bind(C, name="bs2e_slater")
            import :: c_int32_t, c_ptr
            type(c_ptr), value :: h
        end function

        integer(c_int32_t) function bs2e_rk(h, k_first, k_count) bind(C, name="bs2e_rk")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: k_first, k_count
        end function

        integer(c_int32_t) function bs2e_rk_get(h, key, vals) bind(C, name="bs2e_rk_get")
            import :: c_int32_t, c_int64_t, c_double, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), intent(in) :: key(4)
            real(c_double), intent(out) :: vals(*)
        end function

        integer(c_int32_t) function bs2e_set_one_body(h, H1p, n_l, S) bind(C, name="bs2e_set_one_body")
            import :: c_int32_t, c_int64_t, c_double_complex, c_ptr
            type(c_ptr), value :: h
            complex(c_double_complex), intent(in) :: H1p(*)
            integer(c_int64_t), value :: n_l
            complex(c_double_complex), intent(in) :: S(*)
        end function

        integer(c_int32_t) function bs2e_block_count(h, configs, n_config, L, full, nnz_H, nnz_S) &
                bind(C, name="bs2e_block_count")
            import :: c_int32_t, c_int64_t, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, full
            integer(c_int64_t), intent(out) :: nnz_H, nnz_S
        end function

        integer(c_int32_t) function bs2e_block_fill(h, configs, n_config, L, full, H1p, n_l, S, &
                H_index_ptr, H_indices, H_data, S_index_ptr, S_indices, S_data) &
                bind(C, name="bs2e_block_fill")
            import :: c_int32_t, c_int64_t, c_double_complex, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, full
            type(c_ptr), value :: H1p, S          ! c_null_ptr: use bs2e_set_one_body's copy
            integer(c_int64_t), value :: n_l
            integer(c_int64_t), intent(out) :: H_index_ptr(*), H_indices(*)
            complex(c_double_complex), intent(out) :: H_data(*)
            integer(c_int64_t), intent(out) :: S_index_ptr(*), S_indices(*)
            complex(c_double_complex), intent(out) :: S_data(*)
        end function

        ! every symmetry block in one call: configs, H_*, S_* are arrays of
        ! c_loc() addresses (one per block), n_config, L, spin, nnz_* per block
        integer(c_int32_t) function bs2e_blocks_count_all(h, n_blocks, configs, n_config, L, &
                spin, full, nnz_H, nnz_S) bind(C, name="bs2e_blocks_count_all")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: n_blocks, full
            type(c_ptr), intent(in) :: configs(*)
            integer(c_int64_t), intent(in) :: n_config(*), L(*), spin(*)
            integer(c_int64_t), intent(out) :: nnz_H(*), nnz_S(*)
        end function

        integer(c_int32_t) function bs2e_blocks_fill_all(h, n_blocks, configs, n_config, L, &
                spin, full, H_index_ptr, H_indices, H_data, S_index_ptr, S_indices, S_data, &
                out_on_device) bind(C, name="bs2e_blocks_fill_all")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: n_blocks, full, out_on_device
            type(c_ptr), intent(in) :: configs(*)
            integer(c_int64_t), intent(in) :: n_config(*), L(*), spin(*)
            type(c_ptr), intent(in) :: H_index_ptr(*), H_indices(*), H_data(*)
            type(c_ptr), intent(in) :: S_index_ptr(*), S_indices(*), S_data(*)
        end function

        ! rows row_first .. row_first+row_count-1 (0-based first row) of a block,
        ! range-local index_ptr; spin = 0 singlet, 1 triplet
        integer(c_int32_t) function bs2e_block_count_rows(h, configs, n_config, L, spin, full, &
                row_first, row_count, nnz_H, nnz_S) bind(C, name="bs2e_block_count_rows")
            import :: c_int32_t, c_int64_t, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, spin, full, row_first, row_count
            integer(c_int64_t), intent(out) :: nnz_H, nnz_S
        end function

        integer(c_int32_t) function bs2e_block_fill_rows(h, configs, n_config, L, spin, full, &
                row_first, row_count, H_index_ptr, H_indices, H_data, S_index_ptr, S_indices, &
                S_data, out_on_device) bind(C, name="bs2e_block_fill_rows")
            import :: c_int32_t, c_int64_t, c_double_complex, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, spin, full, row_first, row_count
            integer(c_int64_t), intent(out) :: H_index_ptr(*), H_indices(*)
            complex(c_double_complex), intent(out) :: H_data(*)
            integer(c_int64_t), intent(out) :: S_index_ptr(*), S_indices(*)
            complex(c_double_complex), intent(out) :: S_data(*)
            integer(c_int64_t), value :: out_on_device
        end function

        ! n1 bands of a block (rows of every channel with n1 in
        ! [n1_first, n1_first + n1_count)), for blocks larger than memory:
        ! sizes (and, with per_n1, (rows, nnz_H, nnz_S) per n1), then the
        ! band's CSR and its 1-based block rows into host arrays
        ! (out_on_device = 0) or device arrays (1).
        integer(c_int32_t) function bs2e_block_band_count(h, configs, n_config, L, spin, full, &
                n1_first, n1_count, n_rows, nnz_H, nnz_S, per_n1) &
                bind(C, name="bs2e_block_band_count")
            import :: c_int32_t, c_int64_t, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, spin, full, n1_first, n1_count
            integer(c_int64_t), intent(out) :: n_rows, nnz_H, nnz_S
            integer(c_int64_t), intent(out) :: per_n1(*)
        end function

        integer(c_int32_t) function bs2e_block_fill_band(h, configs, n_config, L, spin, full, &
                n1_first, n1_count, rows, H_index_ptr, H_indices, H_data, S_index_ptr, &
                S_indices, S_data, out_on_device) bind(C, name="bs2e_block_fill_band")
            import :: c_int32_t, c_int64_t, c_double_complex, c_ptr, bs2e_config_c
            type(c_ptr), value :: h
            type(bs2e_config_c), intent(in) :: configs(*)
            integer(c_int64_t), value :: n_config, L, spin, full, n1_first, n1_count
            integer(c_int64_t), intent(out) :: rows(*), H_index_ptr(*), H_indices(*)
            complex(c_double_complex), intent(out) :: H_data(*)
            integer(c_int64_t), intent(out) :: S_index_ptr(*), S_indices(*)
            complex(c_double_complex), intent(out) :: S_data(*)
            integer(c_int64_t), value :: out_on_device
        end function

        ! counted blocks the handle keeps (0..16); 0 recounts every block
        integer(c_int32_t) function bs2e_set_block_cache(h, n_blocks) &
                bind(C, name="bs2e_set_block_cache")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: n_blocks
        end function

        ! recreate the handle's stream with a CUDA stream priority (smaller is higher)
        integer(c_int32_t) function bs2e_set_stream_priority(h, priority) &
                bind(C, name="bs2e_set_stream_priority")
            import :: c_int32_t, c_int64_t, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: priority
        end function

        ! CSR_mv (op 0), CSR_T_mv (op 1), CSR_mv_sym (op 2) of a type(CSR_matrix)
        integer(c_int32_t) function bs2e_csr_mv(h, op, n_rows, n_cols, nnz, index_ptr, indices, &
                data, x, y, on_device) bind(C, name="bs2e_csr_mv")
            import :: c_int32_t, c_int64_t, c_double_complex, c_ptr
            type(c_ptr), value :: h
            integer(c_int64_t), value :: op, n_rows, n_cols, nnz
            integer(c_int64_t), intent(in) :: index_ptr(*), indices(*)
            complex(c_double_complex), intent(in) :: data(*), x(*)
            complex(c_double_complex), intent(out) :: y(*)
            integer(c_int64_t), value :: on_device
        end function
    end interface

contains

    ! Turns a non-zero status into error stop with the library's message
    ! (the reference reports failures with stop / error stop, input_tools.f90:938-942).
    subroutine bs2e_check(h, st, where)
        type(c_ptr), intent(in) :: h
        integer(c_int32_t), intent(in) :: st
        character(len=*), intent(in) :: where
        character(kind=c_char) :: buf(1024)
        character(len=1024) :: msg
        integer(c_int32_t) :: ignored
        integer :: i
        if (st == BS2E_OK) return
        msg = ''
        if (c_associated(h)) then
            ignored = bs2e_last_error(h, buf, 1024_c_int64_t)
            do i = 1, 1024
                if (buf(i) == c_null_char) exit
                msg(i:i) = buf(i)
            end do
        end if
        write(6, '(a,a,a,i0,a,a)') 'bs2e error in ', where, ': status ', st, ': ', trim(msg)
        error stop
    end subroutine bs2e_check

    ! type(config) list of one symmetry -> bind(C) records
    subroutine bs2e_pack_configs(configs, packed)
        use orbital_tools, only: config
        type(config), intent(in) :: configs(:)
        type(bs2e_config_c), allocatable, intent(out) :: packed(:)
        integer :: i
        allocate(packed(size(configs)))
        do i = 1, size(configs)
            packed(i)%n1 = configs(i)%n(1)
            packed(i)%n2 = configs(i)%n(2)
            packed(i)%l1 = configs(i)%l(1)
            packed(i)%l2 = configs(i)%l(2)
            packed(i)%eqv = merge(1_c_int64_t, 0_c_int64_t, configs(i)%eqv)
        end do
    end subroutine bs2e_pack_configs
end module bs2e_gpu
