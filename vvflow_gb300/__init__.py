"""GB300-native per-step velocity evaluation for the Viscous Vortex Domains method."""
