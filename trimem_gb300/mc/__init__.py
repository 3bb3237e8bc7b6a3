"""Monte Carlo drivers over ``trimem_gb300.core`` (the reference's
``trimem.mc`` hmc / mesh / evaluators modules) and a device-resident hybrid
HMC + flip driver."""
