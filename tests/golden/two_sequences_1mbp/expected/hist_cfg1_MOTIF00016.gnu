set output "hist_cfg1_MOTIF00016.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-28.2548:9.33746]
set yrange [0:133540]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00016.dat" using 1:2 title 'MOTIF00016 (cfg1)' with boxes
