// How the gas of the nebula decays (values match sol_gas_decrease_type).
#ifndef GASDECREASETYPE_H_
#define GASDECREASETYPE_H_

enum GasDecreaseType { CONSTANT, LINEAR, EXPONENTIAL };

#endif
