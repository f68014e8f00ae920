"""GB300-native SIMPLE hot path of the SYSU_CFD_HEAT finite-volume solver."""
