// Generated by gcchem.hetstate (emit_c). Do not edit.
#pragma once
// rows of the cell-interleaved HetState array (order of the Fortran type)
#define HET_NFIELD 168
#define HET_AVO 0
#define HET_natSurface 1
#define HET_pscBox 2
#define HET_stratBox 3
#define HET_NAEROTYPE 4
#define HET_aClArea 5
#define HET_aClRadi 6
#define HET_aClVol 7
#define HET_aIce 8
#define HET_aLiq 9
#define HET_aWater 10  /* 2 rows */
#define HET_Br_conc_CldA 12
#define HET_Br_conc_CldC 13
#define HET_Br_conc_CldG 14
#define HET_Br_conc_Cld 15
#define HET_Br_conc_SSA 16
#define HET_Br_conc_SSC 17
#define HET_Br_over_Cl_Cld 18
#define HET_Br_over_Cl_SSA 19
#define HET_Br_over_Cl_SSC 20
#define HET_Cl_conc_CldA 21
#define HET_Cl_conc_CldC 22
#define HET_Cl_conc_CldG 23
#define HET_Cl_conc_Cld 24
#define HET_Cl_conc_SSA 25
#define HET_Cl_conc_SSC 26
#define HET_cldFr 27
#define HET_clearFr 28
#define HET_frac_Br_CldA 29
#define HET_frac_Br_CldC 30
#define HET_frac_Br_CldG 31
#define HET_frac_Cl_CldA 32
#define HET_frac_Cl_CldC 33
#define HET_frac_Cl_CldG 34
#define HET_frac_HSO3_aq 35
#define HET_frac_SALACL 36
#define HET_frac_SO3_aq 37
#define HET_fupdateHOBr 38
#define HET_fupdateHOCl 39
#define HET_gamma_HO2 40
#define HET_H2O 41
#define HET_HBr_theta 42
#define HET_HCl_theta 43
#define HET_H_conc_ICl 44
#define HET_H_conc_LCl 45
#define HET_H_conc_SSA 46
#define HET_H_conc_SSC 47
#define HET_H_conc_Sul 48
#define HET_HNO3_theta 49
#define HET_HSO3_aq 50
#define HET_SO3_aq 51
#define HET_HSO3m 52
#define HET_SO3mm 53
#define HET_TSO3_aq 54
#define HET_H_plus 55
#define HET_KHETI_SLA 56  /* 11 rows */
#define HET_HSO4_molal 67
#define HET_NO3_molal 68
#define HET_SO4_molal 69
#define HET_NIT_conc_SSA 70
#define HET_NIT_conc_SSC 71
#define HET_PI 72
#define HET_pHCloud 73
#define HET_pHSSA 74  /* 2 rows */
#define HET_OMOC_POA 76
#define HET_OMOC_OPOA 77
#define HET_qIce 78
#define HET_qLiq 79
#define HET_rIce 80
#define HET_rLiq 81
#define HET_f_Acid_SSA 82
#define HET_f_Acid_SSC 83
#define HET_f_Alk_SSA 84
#define HET_f_Alk_SSC 85
#define HET_SSA_is_Alk 86
#define HET_SSA_is_Acid 87
#define HET_SSC_is_Alk 88
#define HET_SSC_is_Acid 89
#define HET_vAir 90
#define HET_vIce 91
#define HET_vLiq 92
#define HET_wetArea 93  /* 14 rows */
#define HET_xArea 107  /* 14 rows */
#define HET_xH2O 121  /* 14 rows */
#define HET_xRadi 135  /* 14 rows */
#define HET_xVol 149  /* 14 rows */
#define HET_cloudBox 163
#define HET_fracOrgAer 164
#define HET_fracInorgAer 165
#define HET_TurnOffHetRates 166
#define HET_SUNCOS 167
// rows of the cell-interleaved fullchem_SetStateHet input array
#define HETIN_NFIELD 115
#define HETIN_T 0
#define HETIN_CLDF 1
#define HETIN_QI 2
#define HETIN_QL 3
#define HETIN_AIRVOL 4
#define HETIN_AIRDEN 5
#define HETIN_AD 6
#define HETIN_FRLAND 7
#define HETIN_FROCEAN 8
#define HETIN_InStratosphere 9
#define HETIN_aClArea 10
#define HETIN_aClRadi 11
#define HETIN_IsorropAeroH2O 12  /* 2 rows */
#define HETIN_AeroArea 14  /* 14 rows */
#define HETIN_AeroRadi 28  /* 14 rows */
#define HETIN_WetAeroArea 42  /* 14 rows */
#define HETIN_AeroH2O 56  /* 14 rows */
#define HETIN_OMOC_POA 70
#define HETIN_OMOC_OPOA 71
#define HETIN_HSO3_aq 72
#define HETIN_SO3_aq 73
#define HETIN_IsorropBisulfate 74
#define HETIN_IsorropNitrate 75
#define HETIN_IsorropSulfate 76
#define HETIN_IsorropHplus 77
#define HETIN_pHCloud 78
#define HETIN_IsorropAeropH 79  /* 2 rows */
#define HETIN_SALA 81
#define HETIN_SALAAL 82
#define HETIN_SALC 83
#define HETIN_SALCAL 84
#define HETIN_fupdateHOBr 85
#define HETIN_fupdateHOCl 86
#define HETIN_KHETI_SLA 87  /* 11 rows */
#define HETIN_STATE_PSC 98
#define HETIN_SUNCOS 99
#define HETIN_PMID_DRY 100
#define HETIN_NH4 101
#define HETIN_NH3 102
#define HETIN_DSTbin 103  /* 7 rows */
#define HETIN_pFe 110
#define HETIN_OMEGA 111
#define HETIN_U 112
#define HETIN_V 113
#define HETIN_IsWater 114
// KPP species read by fullchem_SetStateHet and fullchem_SulfurAqChem, in the order of the index table
#define HSS_SO2 0
#define HSS_HNO3 1
#define HSS_HCl 2
#define HSS_HBr 3
#define HSS_BrSALA 4
#define HSS_BrSALC 5
#define HSS_SALACL 6
#define HSS_SALCCL 7
#define HSS_NIT 8
#define HSS_NITs 9
#define HSS_SO4 10
#define HSS_SALAAL 11
#define HSS_SALCAL 12
#define HSS_O3 13
#define HSS_H2O2 14
#define HSS_CH2O 15
#define HSS_SO4s 16
#define HSS_HMS 17
#define HSS_HCOOH 18
#define HSS_ACTA 19
#define HSS_HOCl 20
#define HSS_HOBr 21
#define HSS_N 22
// MW_g of the non-KPP species SET_SO2 reads (species database)
#define HSS_MW_DSTbin1 29.0
#define HSS_MW_pFe 55.85
#define HSS_MW_SALA 31.4
#define HSS_MW_SALC 31.4
#define HSS_MW_SO4 96.06
