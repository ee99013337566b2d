set output "hist_cfg1_MOTIF00023.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-32.1134:9.83792]
set yrange [0:122504]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00023.dat" using 1:2 title 'MOTIF00023 (cfg1)' with boxes
