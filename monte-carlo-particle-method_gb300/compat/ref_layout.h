// ref_layout.h -- written by make_layout.py: byte offsets and sizes of the
// fields the drop-in routines use in the reference's structs GAS, BOX and
// CELLS (src/cpp_headers.h:145-347), measured by compiling offsetof()
// against the reference's header.  MCPM_REF_<struct>_<field> is
// "offset, size" in bytes.  Do not edit: run make_layout.py again.
#pragma once
#define MCPM_REF_SIZEOF_GAS 872
#define MCPM_REF_GAS_N 416, 8
#define MCPM_REF_GAS_sigma 400, 8
#define MCPM_REF_GAS_m 432, 8
#define MCPM_REF_GAS_kb 488, 8
#define MCPM_REF_GAS_n 408, 8
#define MCPM_REF_GAS_Fn 688, 8
#define MCPM_REF_GAS_T0 464, 8
#define MCPM_REF_GAS_mu 552, 8
#define MCPM_REF_GAS_visp 808, 8
#define MCPM_REF_GAS_b 720, 8
#define MCPM_REF_GAS_delta_t 472, 8
#define MCPM_REF_GAS_phi 360, 8
#define MCPM_REF_GAS_eqdist 368, 8
#define MCPM_REF_GAS_ast 384, 8
#define MCPM_REF_GAS_bst 392, 8
#define MCPM_REF_GAS_crref 816, 8
#define MCPM_REF_GAS_model 616, 32
#define MCPM_REF_GAS_long_range 856, 4
#define MCPM_REF_GAS_Tc 208, 8
#define MCPM_REF_GAS_Th 216, 8
#define MCPM_REF_GAS_n_ratio 860, 4
#define MCPM_REF_GAS_T 456, 8
#define MCPM_REF_SIZEOF_BOX 816
#define MCPM_REF_BOX_N 536, 12
#define MCPM_REF_BOX_Len 416, 24
#define MCPM_REF_BOX_delta_dim 440, 24
#define MCPM_REF_BOX_direction 788, 12
#define MCPM_REF_BOX_problem 580, 4
#define MCPM_REF_BOX_T_wall_1 640, 8
#define MCPM_REF_BOX_T_wall_2 648, 8
#define MCPM_REF_BOX_T_wall_3 656, 8
#define MCPM_REF_BOX_T_wall_4 664, 8
#define MCPM_REF_BOX_U_wall_1 584, 8
#define MCPM_REF_BOX_U_wall_2 592, 8
#define MCPM_REF_BOX_U_wall_3 600, 8
#define MCPM_REF_BOX_U_wall_4 608, 8
#define MCPM_REF_BOX_step 800, 4
#define MCPM_REF_BOX_thermc 48, 8
#define MCPM_REF_BOX_thermh 56, 8
#define MCPM_REF_BOX_file_name 752, 32
#define MCPM_REF_SIZEOF_CELLS 1984
#define MCPM_REF_CELLS_num_inside 376, 4
#define MCPM_REF_CELLS_indices_inside 368, 8
#define MCPM_REF_CELLS_weight 280, 8
#define MCPM_REF_CELLS_U_space 552, 24
#define MCPM_REF_CELLS_PIJ 616, 48
#define MCPM_REF_CELLS_M3 760, 80
#define MCPM_REF_CELLS_M4 664, 48
#define MCPM_REF_CELLS_M5 712, 24
#define MCPM_REF_CELLS_Q 736, 24
#define MCPM_REF_CELLS_DM2 840, 8
#define MCPM_REF_CELLS_DM4 848, 8
#define MCPM_REF_CELLS_Mp 1888, 24
#define MCPM_REF_CELLS_T 576, 8
#define MCPM_REF_CELLS_n 584, 8
#define MCPM_REF_CELLS_gamma_st 928, 8
#define MCPM_REF_CELLS_Lambda 1944, 8
#define MCPM_REF_CELLS_c 856, 48
#define MCPM_REF_CELLS_gamma 904, 24
#define MCPM_REF_CELLS_alpha 384, 72
#define MCPM_REF_CELLS_beta 528, 24
#define MCPM_REF_CELLS_phi 1912, 24
#define MCPM_REF_CELLS_F2 1968, 8
#define MCPM_REF_CELLS_omega_max 1936, 8
#define MCPM_REF_CELLS_crm 936, 8
#define MCPM_REF_CELLS_divU 48, 8
#define MCPM_REF_CELLS_n_smooth 272, 8
#define MCPM_REF_CELLS_dn2 256, 8
#define MCPM_REF_CELLS_dn3 264, 8
#define MCPM_REF_CELLS_n_ratio 72, 4
#define MCPM_REF_CELLS_p_m 0, 8
