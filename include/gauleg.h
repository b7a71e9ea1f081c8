/* gauleg.h -- Gauss-Legendre nodes and weights on [x1,x2] (reference com_src/gauleg.h). */
#ifndef GAULEG_H_
#define GAULEG_H_
void gauleg(double x1, double x2, double x[], double w[], int n);
#endif
