"""halign_gb300: GB300-native align-to-center path of HAlign-4 (package directory ``halign-4_gb300``)."""
