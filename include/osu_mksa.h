/*
 * osu_mksa.h -- conversion from the normalised unit system (c0 = mu0 = 1) to
 * MKSA, used only for printing (reference com_src/osu_mksa.h).
 */
#ifndef OSU_MKSA_H
#define OSU_MKSA_H
double OSUtoMKSA_length(double l);
double OSUtoMKSA_Power_per_unit_area(double p);
double OSUtoMKSA_Force(double f);
double OSUtoMKSA_Torque(double n);
double OSUtoMKSA_Power(double p);
double OSUtoMKSA_power(double p);
#endif
