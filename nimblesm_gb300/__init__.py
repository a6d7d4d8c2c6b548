"""GB300-native explicit hex8 / neo-Hookean transient-dynamics engine."""
